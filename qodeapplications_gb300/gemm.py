"""Host-side builder of grouped-GEMM task tables for libxrh (xrh_gemm_task / xrh_gemm_segment).

A task is one output block; its segments are the contractions summed into it (K
concatenation).  Tables are built once per plan with the device addresses of persistent
buffers and uploaded once, so every later launch is a single call (CUDA-graph safe).
"""
import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import SEGMENT_DTYPE, TASK_DTYPE, call, ptr, stream_ptr

FP64_TILE = 64


class GroupedGemm:
    def __init__(self, device="cuda", precision="fp64"):
        self.device = torch.device(device)
        self.precision = _lib.PRECISIONS[precision]
        self._tasks = []
        self._segs = []
        self._keep = []          # tensors whose addresses are in the tables
        self.tasks_dev = None
        self.segs_dev = None
        self.total_tiles = 0
        self.flops = 0.0         # algorithmic FLOPs of one launch (2*M*N*K per segment)

    def add(self, M, N, segments, C, ldc, mode=0, splitk=1, maps=None, DA=None, DB=None, batch=1, sC=0):
        """segments: list of (A, lda, B, ldb, K, alpha[, flags, sA, sB]) with A, B torch CUDA
        float64 tensors.  flags bit 0: A stored [k][m] (else [m][k]); bit 1: B stored [k][n]
        (else [n][k]).  batch > 1 repeats the problem with pointer strides sA, sB, sC.
        maps: (rowA, colA, rowB, colB, diagA, diagB) for mode 2."""
        if M <= 0 or N <= 0 or batch <= 0:
            return
        seg_begin = len(self._segs)
        for seg in segments:
            A, lda, B, ldb, K, alpha = seg[:6]
            flags, sA, sB = (seg[6], seg[7], seg[8]) if len(seg) > 6 else (0, 0, 0)
            assert A.dtype == torch.float64 and B.dtype == torch.float64 and A.is_cuda and B.is_cuda
            assert A.is_contiguous() and B.is_contiguous()
            a_need = (batch - 1) * sA + ((K - 1) * lda + M if flags & 1 else (M - 1) * lda + K)
            b_need = (batch - 1) * sB + ((K - 1) * ldb + N if flags & 2 else (N - 1) * ldb + K)
            assert A.numel() >= a_need and B.numel() >= b_need, "operand too small"
            self._segs.append((A.data_ptr(), B.data_ptr(), lda, ldb, K, float(alpha), flags, sA, sB))
            self._keep += [A, B]
            self.flops += 2.0 * M * N * K * batch
        if mode != 2:
            assert C.numel() >= (batch - 1) * sC + (M - 1) * ldc + N, "output too small"
        t = dict(M=M, N=N, seg_begin=seg_begin, seg_count=len(segments), mode=mode, splitk=splitk,
                 C=C.data_ptr(), ldc=ldc, batch=batch, sC=sC)
        self._keep.append(C)
        if mode == 2:
            rowA, colA, rowB, colB, diagA, diagB = maps
            for nm, tt in zip(("rowA", "colA", "rowB", "colB", "diagA", "diagB"), maps):
                t[nm] = tt.data_ptr()
                self._keep.append(tt)
            t["DA"] = DA.data_ptr() if DA is not None else 0
            t["DB"] = DB.data_ptr() if DB is not None else 0
            self._keep += [x for x in (DA, DB) if x is not None]
        self._tasks.append(t)

    def finalize(self, tile=FP64_TILE):
        tasks = np.zeros(len(self._tasks), dtype=TASK_DTYPE)
        begin = 0
        for i, t in enumerate(self._tasks):
            for k, v in t.items():
                tasks[i][k] = v
            tasks[i]["tile_begin"] = begin
            begin += ((t["M"] + tile - 1) // tile) * ((t["N"] + tile - 1) // tile) * t["splitk"] * t["batch"]
        self.total_tiles = begin
        segs = np.zeros(len(self._segs), dtype=SEGMENT_DTYPE)
        for i, s in enumerate(self._segs):
            segs[i] = s
        self.tasks_dev = torch.from_numpy(tasks.view(np.uint8).copy()).to(self.device)
        self.segs_dev = torch.from_numpy(segs.view(np.uint8).copy()).to(self.device) if len(segs) else \
            torch.zeros(SEGMENT_DTYPE.itemsize, dtype=torch.uint8, device=self.device)
        self.n_tasks = len(self._tasks)
        return self

    def run(self, stream=None):
        if self.n_tasks == 0:
            return
        call("xrh_gemm_simt_grouped", self.precision, _lib.ptr(self.tasks_dev), self.n_tasks, self.total_tiles,
             _lib.ptr(self.segs_dev), stream_ptr(stream))


TC_TASK_DTYPE = np.dtype([("M", np.int64), ("N", np.int64), ("seg_begin", np.int64), ("seg_count", np.int64),
                          ("mode", np.int64), ("splitk", np.int64), ("tile_begin", np.int64), ("bn", np.int64),
                          ("C", np.uint64), ("ldc", np.int64), ("rowA", np.uint64), ("colA", np.uint64),
                          ("rowB", np.uint64), ("colB", np.uint64), ("DA", np.uint64), ("DB", np.uint64),
                          ("diagA", np.uint64), ("diagB", np.uint64)])
TC_SEG_DTYPE = np.dtype([("tmA", np.int64), ("tmB", np.int64), ("kchunks", np.int64), ("negate", np.int64)])
assert TC_TASK_DTYPE.itemsize == 144 and TC_SEG_DTYPE.itemsize == 32
TC_BM = 128


class SplitRegistry:
    """hi/lo split copies of FP64 operands for the tensor-core path, and their TMA maps.

    Every operand tensor is split once per build (split(group)); its two 128-byte TMA
    descriptors per box height are encoded once on the host and uploaded with upload()."""

    def __init__(self, precision, device="cuda"):
        self.prec = _lib.PRECISIONS[precision]
        assert self.prec in (_lib.BF16X3, _lib.TF32X3)
        self.kch = 64 if self.prec == _lib.BF16X3 else 32
        self.dtype = torch.bfloat16 if self.prec == _lib.BF16X3 else torch.int32
        self.device = torch.device(device)
        self.ops = {}        # data_ptr -> dict
        self.maps = []       # host byte strings, 128 B each
        self.map_index = {}
        self.maps_dev = None
        self._split_tables = {}

    def operand(self, t, rows, K, ld, group="in"):
        key = t.data_ptr()
        if key not in self.ops:
            self._split_tables.pop(group, None)      # rebuilt at the group's next split
            Kp = ((K + self.kch - 1) // self.kch) * self.kch
            hi = torch.zeros((rows, Kp), dtype=self.dtype, device=self.device)
            lo = torch.zeros((rows, Kp), dtype=self.dtype, device=self.device)
            self.ops[key] = dict(src=t, rows=rows, K=K, ld=ld, Kp=Kp, hi=hi, lo=lo, group=group)
        op = self.ops[key]
        assert op["rows"] == rows and op["K"] == K and op["ld"] == ld, "operand registered with another shape"
        return op

    def map_for(self, t, box_rows):
        key = (t.data_ptr(), box_rows)
        if key not in self.map_index:
            op = self.ops[t.data_ptr()]
            idx = len(self.maps)
            for part in ("hi", "lo"):
                buf = ctypes.create_string_buffer(128)
                call("xrh_tc_encode_map", self.prec, ptr(op[part]), op["rows"], op["Kp"], box_rows, buf)
                self.maps.append(buf.raw)
            self.map_index[key] = idx
        return self.map_index[key]

    def upload(self):
        raw = b"".join(self.maps) if self.maps else bytes(128)
        self.maps_dev = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(self.device)
        assert self.maps_dev.data_ptr() % 64 == 0

    def split(self, group, stream=None):
        """Split every operand of `group` in one launch (task table built on first use and again
        after an operand joins the group; not during a graph capture)."""
        s = stream_ptr(stream)
        if group not in self._split_tables:
            ops = [op for op in self.ops.values() if op["group"] == group]
            tasks = np.zeros(len(ops), dtype=_lib.SPLIT_TASK_DTYPE)
            begin = 0
            for i, op in enumerate(ops):
                t = tasks[i]
                t["src"], t["hi"], t["lo"] = op["src"].data_ptr(), op["hi"].data_ptr(), op["lo"].data_ptr()
                t["rows"], t["K"], t["ld"], t["Kp"], t["group_begin"] = op["rows"], op["K"], op["ld"], op["Kp"], begin
                begin += op["rows"] * op["Kp"] // 4
            dev = torch.from_numpy(tasks.view(np.uint8).copy()).to(self.device) if len(ops) else None
            self._split_tables[group] = (dev, len(ops), begin)
        dev, n, total = self._split_tables[group]
        if n:
            call("xrh_split_grouped", self.prec, ptr(dev), n, total, s)


_TUNE_CACHE = {}


class TCGroupedGemm:
    """Task tables for xrh_gemm_tc_grouped (split precision on tcgen05).

    Tile policy: each task gets an N tile bn in {32, 64, 128} (capped by the policy) and, for
    accumulating tasks (mode 1), a split-K factor kc_total // div (1..32).  autotune() times
    every (cap, div) pair on the device with CUDA events and keeps the fastest; results are
    cached per problem signature, so later plans of the same shapes reuse them."""

    BN_CAPS = (128, 64, 32)
    SK_DIVS = (16, 4, 8, 32)

    def __init__(self, registry):
        self.reg = registry
        self.device = registry.device
        self._logical = []
        self.flops = 0.0
        self.policy = (128, 16)
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.tuning = None

    def add(self, M, N, segments, C, ldc, mode=0, splitk=None, maps=None, DA=None, DB=None, groups=None):
        if M <= 0 or N <= 0:
            return
        segs = []
        for i, (A, lda, B, ldb, K, alpha) in enumerate(segments):
            assert abs(abs(alpha) - 1.0) < 1e-15, "tensor-core segments take alpha = +-1 (fold scales into operands)"
            ga, gb = (groups[i] if groups else ("in", "in"))
            self.reg.operand(A, M, K, lda, ga)
            self.reg.operand(B, N, K, ldb, gb)
            segs.append((A, B, 1 if alpha < 0 else 0))
            self.flops += 2.0 * M * N * K
        self._logical.append(dict(M=M, N=N, segs=segs, C=C, ldc=ldc, mode=mode, splitk=splitk, maps=maps,
                                  DA=DA, DB=DB))

    def _bn(self, N, cap):
        bn = 32 if N <= 32 else (64 if N <= 64 else 128)
        return min(bn, cap)

    def _materialize(self, policy):
        cap, div = policy
        tasks = np.zeros(len(self._logical), dtype=TC_TASK_DTYPE)
        seg_rows = []
        begin = 0
        for i, L in enumerate(self._logical):
            bn = self._bn(L["N"], cap)
            seg_begin = len(seg_rows)
            kc_total = 0
            for (A, B, neg) in L["segs"]:
                kch = self.reg.ops[A.data_ptr()]["Kp"] // self.reg.kch
                seg_rows.append((self.reg.map_for(A, TC_BM), self.reg.map_for(B, bn), kch, neg))
                kc_total += kch
            sk = L["splitk"]
            if sk is None:
                sk = int(max(1, min(32, kc_total // div))) if L["mode"] == 1 else 1
            t = tasks[i]
            t["M"], t["N"], t["seg_begin"], t["seg_count"] = L["M"], L["N"], seg_begin, len(L["segs"])
            t["mode"], t["splitk"], t["bn"], t["C"], t["ldc"] = L["mode"], sk, bn, L["C"].data_ptr(), L["ldc"]
            if L["mode"] == 2:
                for nm, tt in zip(("rowA", "colA", "rowB", "colB", "diagA", "diagB"), L["maps"]):
                    t[nm] = tt.data_ptr()
                t["DA"] = L["DA"].data_ptr() if L["DA"] is not None else 0
                t["DB"] = L["DB"].data_ptr() if L["DB"] is not None else 0
            t["tile_begin"] = begin
            begin += ((L["M"] + TC_BM - 1) // TC_BM) * ((L["N"] + bn - 1) // bn) * sk
        segs = np.zeros(max(len(seg_rows), 1), dtype=TC_SEG_DTYPE)
        for i, r in enumerate(seg_rows):
            segs[i] = r
        return tasks, segs, begin

    def finalize(self, policy=None):
        """Build and upload the task tables for a policy (default: the current one).  The
        registry's maps must be uploaded (again) when this adds a box height: finalize
        does it itself when needed."""
        if policy is not None:
            self.policy = policy
        n_maps = len(self.reg.maps)
        tasks, segs, total = self._materialize(self.policy)
        if len(self.reg.maps) != n_maps or self.reg.maps_dev is None:
            self.reg.upload()
        self.total_tiles = total
        self.tasks_dev = torch.from_numpy(tasks.view(np.uint8).copy()).to(self.device)
        self.segs_dev = torch.from_numpy(segs.view(np.uint8).copy()).to(self.device)
        self.n_tasks = len(self._logical)
        return self

    def signature(self):
        return (self.reg.prec,) + tuple((L["M"], L["N"], L["mode"], L["splitk"],
                                         tuple(self.reg.ops[A.data_ptr()]["Kp"] for (A, _, _) in L["segs"]))
                                        for L in self._logical)

    def autotune(self, reps=3):
        """Time every tile policy on the device (the launch writes its own outputs; call it
        before the first build, which clears accumulation targets itself) and keep the best."""
        if not self._logical:
            return self
        key = self.signature()
        if key in _TUNE_CACHE:
            return self.finalize(_TUNE_CACHE[key])
        has_acc = any(L["mode"] == 1 and L["splitk"] is None for L in self._logical)
        caps = [c for c in self.BN_CAPS if c == 128 or any(L["N"] > c for L in self._logical)]
        divs = self.SK_DIVS if has_acc else self.SK_DIVS[:1]
        results = []
        for cap in caps:
            for div in divs:
                self.finalize((cap, div))
                self.run()
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(reps):
                    self.run()
                e1.record()
                torch.cuda.synchronize()
                results.append((e0.elapsed_time(e1) / reps, (cap, div)))
        self.check()
        results.sort()
        self.tuning = [(p, round(ms, 4)) for ms, p in results]
        _TUNE_CACHE[key] = results[0][1]
        return self.finalize(results[0][1])

    def run(self, stream=None):
        if self.n_tasks == 0:
            return
        call("xrh_gemm_tc_grouped", self.reg.prec, ptr(self.tasks_dev), self.n_tasks, self.total_tiles,
             ptr(self.segs_dev), ptr(self.reg.maps_dev), ptr(self.status), stream_ptr(stream))

    def check(self):
        st = int(self.status.item())
        if st != 0:
            raise _lib.XRHError(f"tensor-core GEMM reported status {st} ({_lib.lib().xrh_status_string(st).decode()})")

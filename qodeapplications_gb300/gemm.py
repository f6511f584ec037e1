"""Host-side builder of grouped-GEMM task tables for libxrh (xrh_gemm_task / xrh_gemm_segment).

A task is one output block; its segments are the contractions summed into it (K
concatenation).  Tables are built once per plan with the device addresses of persistent
buffers and uploaded once, so every later launch is a single call (CUDA-graph safe).
"""
import numpy as np
import torch

from . import _lib
from ._lib import SEGMENT_DTYPE, TASK_DTYPE, call, stream_ptr

FP64_TILE = 64


class GroupedGemm:
    def __init__(self, device="cuda"):
        self.device = torch.device(device)
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
        call("xrh_gemm_fp64_grouped", _lib.ptr(self.tasks_dev), self.n_tasks, self.total_tiles,
             _lib.ptr(self.segs_dev), stream_ptr(stream))

"""ctypes binding of libxrh.so (include/xrh.h).

The library is built in-tree by qodeapplications_gb300/build.py.  There is no fallback:
if the shared library is missing or a call returns an error status, an XRHError is raised.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libxrh.so")

XRH_OK, XRH_ERR_ARG, XRH_ERR_CUDA, XRH_ERR_UNSUPPORTED, XRH_ERR_TIMEOUT, XRH_ERR_CAPACITY = range(6)
FP64, FP32, BF16X3, TF32X3 = 0, 1, 2, 3
PRECISIONS = {"fp64": FP64, "fp32": FP32, "bf16x3": BF16X3, "tf32x3": TF32X3}


class XRHError(RuntimeError):
    pass


_i32, _i64, _vp, _dbl = ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_double

_SIGS = {
    "xrh_abi_version": (_i32, []),
    "xrh_density_accumulate_f32_grouped": (_i32, [_vp, _i32, _i64, _i32, _i32, _vp]),
    "xrh_density_accumulate_f32_units": (_i32, [_vp, _i32, _vp, _i64, _i32, _vp]),
    "xrh_density_adjoint_f32_grouped": (_i32, [_vp, _i32, _i64, _i32, _i32, _vp]),
    "xrh_density_adjoint_f32_units": (_i32, [_vp, _i32, _vp, _i64, _i32, _i32, _vp]),
    "xrh_mirror_density": (_i32, [_i32, _i32, _i32, _i32, _vp, _vp, _i32, _vp]),
    "xrh_density_adjoint_tc_grouped": (_i32, [_vp, _i32, _i64, _vp, _vp]),
    "xrh_lanczos_small": (_i32, [_i32, _i32, _vp, _i64, _vp, _vp, _vp, _vp, _vp]),
    "xrh_lanczos_coop_work": (_i64, [_i32]),
    "xrh_lanczos_cluster": (_i32, [_i32, _i32, _vp, _i64, _vp, _vp, _vp, _vp, _i32, _vp]),
    "xrh_lanczos_cluster_fits": (_i32, [_i32, _i32, _i32]),
    "xrh_lanczos_coop": (_i32, [_i64, _i32, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _i64, _vp, _vp]),
    "xrh_lanczos_coop_bounded": (_i32, [_i64, _i32, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _i64, _vp, _i64, _vp]),
    "xrh_state_ctas": (_i32, [_i64]),
    "xrh_abt_ctas": (_i32, [_i64]),
    "xrh_split_grouped": (_i32, [_i32, _vp, _i32, _i64, _vp]),
    "xrh_gemv_rows_grouped": (_i32, [_vp, _i32, _i64, _vp]),
    "xrh_abt_grouped": (_i32, [_i32, _vp, _i32, _i64, _vp]),
    "xrh_coeff_stage": (_i32, [_vp, _i32, _i64, _vp]),
    "xrh_transpose_grouped": (_i32, [_vp, _i32, _i64, _vp]),
    "xrh_mirror_grouped": (_i32, [_vp, _i32, _i64, _vp]),
    "xrh_orbital_terms": (_i32, [_vp, _vp, _vp, _i32, _vp]),
    "xrh_pair_grouped": (_i32, [_i32, _vp, _i32, _i64, _vp]),
    "xrh_gram_grouped": (_i32, [_vp, _i32, _i64, _i32, _vp]),
    "xrh_tangent_step": (_i32, [_vp, _i32, _i64, _dbl, _vp, _vp]),
    "xrh_inv_sqrt_small": (_i32, [_vp, _i32, _i32, _vp]),
    "xrh_left_multiply": (_i32, [_vp, _i32, _i64, _vp]),
    "xrh_abt_small": (_i32, [_i32, _i32, _i32, _i64, _vp, _i64, _vp, _i64, _dbl, _vp, _vp]),
    "xrh_pair_scatter": (_i32, [_i64, _vp, _vp, _vp, _vp, _i32, _vp, _vp, _vp]),
    "xrh_im_scatter": (_i32, [_i64, _vp, _vp, _vp, _vp, _vp, _i32, _i64, _i32, _vp, _vp, _vp]),
    "xrh_im_expand": (_i32, [_i32, _i32, _i64, _vp, _vp, _vp, _i32, _i32, _vp, _vp, _vp]),
    "xrh_im_fold": (_i32, [_i32, _i32, _i64, _i32, _i32, _vp, _vp, _vp, _vp, _vp]),
    "xrh_im_gather": (_i32, [_i32, _vp, _vp, _vp, _vp, _i32, _i64, _i32, _vp, _vp, _vp]),
    "xrh_pair_gather": (_i32, [_i32, _vp, _vp, _vp, _vp, _i32, _vp, _vp, _vp]),
    "xrh_status_string": (ctypes.c_char_p, [_i32]),
    "xrh_last_cuda_error": (_i32, []),
    "xrh_couplings_count": (_i32, [_i32, _i32, _i32, _vp, _i32, _vp, _vp, _i32, _vp, _vp]),
    "xrh_couplings_fill": (_i32, [_i32, _i32, _i32, _vp, _i32, _vp, _vp, _i32, _vp, _vp, _vp, _vp, _vp, _vp]),
    "xrh_density_accumulate": (_i32, [_i32, _i64, _vp, _vp, _vp, _vp, _vp, _i32, _vp, _i32, _vp, _vp]),
    "xrh_transpose": (_i32, [_vp, _i64, _i64, _vp, _vp]),
    "xrh_density_accumulate_f32": (_i32, [_i64, _i32, _vp, _vp, _vp, _vp, _vp, _i32, _vp, _i32, _vp, _vp]),
    "xrh_density_build_noalloc": (_i32, [_i32, _i64, _vp, _vp, _vp, _vp, _vp, _i32, _vp, _i32, _vp, _vp]),
    "xrh_sigma2e": (_i32, [_i32, _i32, _vp, _vp, _i32, _vp, _vp, _i32, _vp, _i64, _vp, _vp, _i32, _vp, _vp]),
    "xrh_gemm_fp64_grouped": (_i32, [_vp, _i32, _i64, _vp, _vp]),
    "xrh_gemm_simt_grouped": (_i32, [_i32, _vp, _i32, _i64, _vp, _vp]),
    "xrh_gemv_rows": (_i32, [_i64, _i64, _vp, _i64, _vp, _dbl, _dbl, _vp, _vp]),
    "xrh_gemv_cols": (_i32, [_i64, _i64, _vp, _i64, _vp, _dbl, _vp, _vp]),
    "xrh_gemv_split_work": (_i64, [_i64, _i64]),
    "xrh_gemv_rows_split": (_i32, [_i64, _i64, _vp, _i64, _vp, _dbl, _dbl, _vp, _vp, _i64, _vp]),
    "xrh_lanczos_normalize_split": (_i32, [_i64, _vp, _vp, _vp, _vp, _i64, _vp]),
    "xrh_lanczos_normalize": (_i32, [_i64, _vp, _vp, _vp, _vp]),
    "xrh_density_adjoint": (_i32, [_i32, _i64, _vp, _vp, _vp, _vp, _vp, _i32, _vp, _i32, _vp, _vp, _vp, _vp]),
    "xrh_ccaa_weighted": (_i32, [_i32, _i32, _vp, _i32, _vp, _vp, _i32, _vp, _i64, _vp, _vp, _vp, _i32, _vp, _vp]),
    "xrh_tc_chunk_elems": (_i32, [_i32]),
    "xrh_split_operand": (_i32, [_i32, _vp, _i64, _i64, _i64, _i64, _vp, _vp, _vp]),
    "xrh_tc_encode_map": (_i32, [_i32, _vp, _i64, _i64, _i32, _vp]),
    "xrh_gemm_tc_grouped": (_i32, [_i32, _vp, _i32, _i64, _vp, _vp, _vp, _vp]),
    "xrh_inverse_small": (_i32, [_i32, _vp, _i64, _vp, _i64, _vp, _vp]),
    "xrh_expm_small": (_i32, [_i32, _vp, _i64, _vp, _i64, _vp]),
    "xrh_spin_block": (_i32, [_i32, _vp, _vp, _vp, _i64, _vp, _i64, _vp]),
    "xrh_gather_submatrix": (_i32, [_i32, _vp, _vp, _i64, _vp, _i64, _vp]),
    "xrh_zero": (_i32, [_vp, _i64, _vp]),
    "xrh_index_move": (_i32, [_i64, _vp, _vp, _vp, _i32, _vp]),
    "xrh_f64_to_f32": (_i32, [_i64, _vp, _vp, _vp]),
    "xrh_mirror_ctas": (_i64, [_i32, _i32]),
    "xrh_antisym_rows": (_i32, [_vp, _i32, _i64, _vp]),
    "xrh_add_mixed": (_i32, [_i64, _dbl, _vp, _vp, _vp, _vp]),
    "xrh_spin_sum_antisym": (_i32, [_i32, _i32, _vp, _vp, _i64, _vp, _vp]),
    "xrh_small_mm_grouped": (_i32, [_vp, _i32, _i64, _vp]),
    "xrh_permute_grouped": (_i32, [_vp, _i32, _i64, _vp]),
    "xrh_gather_sum": (_i32, [_i64, _vp, _vp, _i32, _vp]),
}
_OPTIONAL = {}

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise XRHError(f"{LIB_PATH} is missing: build it with `python -m qodeapplications_gb300.build` "
                           "(there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in list(_SIGS.items()) + list(_OPTIONAL.items()):
            if not hasattr(L, name):
                if name in _OPTIONAL:
                    continue
                raise XRHError(f"{LIB_PATH} does not export {name}")
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def register(name, restype, argtypes):
    """Declare an additional exported symbol (used by modules that add entry points)."""
    _SIGS[name] = (restype, argtypes)
    if _lib is not None:
        f = getattr(_lib, name)
        f.restype = restype
        f.argtypes = argtypes


class LaunchCounter:
    """Counts library calls that launch a kernel (the gpu_launches figure): every entry point
    except the host-only ones below launches one kernel of this library (those in `multi` the
    number given)."""
    multi = {"xrh_orbital_terms": 2, "xrh_gemv_rows_split": 2, "xrh_lanczos_normalize_split": 2}
    host_only = {"xrh_abi_version", "xrh_status_string", "xrh_last_cuda_error", "xrh_tc_chunk_elems", "xrh_zero",
                 "xrh_tc_encode_map", "xrh_state_ctas", "xrh_abt_ctas", "xrh_lanczos_coop_work",
                 "xrh_lanczos_cluster_fits", "xrh_gemv_split_work", "xrh_mirror_ctas"}
    count = 0


def call(name, *args):
    """Call one ABI function; raise XRHError on a non-zero status."""
    if name not in LaunchCounter.host_only:
        LaunchCounter.count += LaunchCounter.multi.get(name, 1)
    st = getattr(lib(), name)(*args)
    if st != XRH_OK:
        msg = lib().xrh_status_string(st).decode()
        raise XRHError(f"{name} failed: {msg} (status {st}, cuda error {lib().xrh_last_cuda_error()})")


def ptr(t):
    """Device (or host) address of a torch tensor, or None."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_ptr(stream=None):
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    return ctypes.c_void_p(s.cuda_stream)


def op_code(op):
    code = len(op)
    for i, ch in enumerate(op):
        if ch == "c":
            code |= 1 << (4 + i)
    return code


# numpy mirrors of the ABI structs (field order and sizes match include/xrh.h)
SEGMENT_DTYPE = np.dtype([("A", np.uint64), ("B", np.uint64), ("lda", np.int64), ("ldb", np.int64),
                          ("K", np.int64), ("alpha", np.float64), ("flags", np.int64), ("sA", np.int64),
                          ("sB", np.int64)])
DENS_ADJ_TASK_DTYPE = np.dtype([("idx_ptr", np.uint64), ("P", np.uint64), ("Q", np.uint64), ("sign", np.uint64),
                                ("zb32", np.uint64), ("zk32", np.uint64), ("gT", np.uint64), ("gzb", np.uint64),
                                ("gzk", np.uint64), ("K", np.int64), ("nb", np.int32), ("nk", np.int32),
                                ("cta_begin", np.int64)])
assert DENS_ADJ_TASK_DTYPE.itemsize == 96
DENS_ADJ_TC_TASK_DTYPE = np.dtype([("idx_ptr", np.uint64), ("P", np.uint64), ("Q", np.uint64), ("sign", np.uint64),
                                   ("zbh", np.uint64), ("zbl", np.uint64), ("zkh", np.uint64), ("zkl", np.uint64),
                                   ("gT", np.uint64), ("gzb", np.uint64), ("gzk", np.uint64), ("K", np.int64),
                                   ("nb", np.int32), ("nk", np.int32), ("cta_begin", np.int64)])
assert DENS_ADJ_TC_TASK_DTYPE.itemsize == 112
DENS_TASK_DTYPE = np.dtype([("idx_ptr", np.uint64), ("P", np.uint64), ("Q", np.uint64), ("sign", np.uint64),
                            ("zb32", np.uint64), ("zk32", np.uint64), ("rhoT", np.uint64), ("K", np.int64),
                            ("nb", np.int32), ("nk", np.int32), ("splits", np.int32), ("reserved", np.int32),
                            ("cta_begin", np.int64)])
assert DENS_TASK_DTYPE.itemsize == 88
PAIR_TASK_DTYPE = np.dtype([("X", np.uint64), ("xptr", np.uint64), ("off", np.uint64), ("sign", np.uint64),
                            ("stride", np.uint64), ("src", np.uint64), ("dst", np.uint64), ("count", np.int64),
                            ("n", np.int64)])
assert PAIR_TASK_DTYPE.itemsize == 72
ORBITAL_INPUTS_DTYPE = np.dtype([("gw", np.uint64), ("h1", np.uint64, 2), ("cca", np.uint64, 2),
                                 ("caa", np.uint64, 2), ("cc", np.uint64, 2), ("mono1", np.uint64, 2),
                                 ("gamma64", np.uint64, 2), ("gamma32", np.uint64, 2), ("N0", np.int32),
                                 ("N1", np.int32)])
assert ORBITAL_INPUTS_DTYPE.itemsize == 128
MIRROR_TASK_DTYPE = np.dtype([("src", np.uint64), ("dst", np.uint64), ("na", np.int32), ("nb", np.int32),
                              ("N", np.int32), ("L", np.int32), ("accumulate", np.int32), ("reserved", np.int32),
                              ("cta_begin", np.int64)])
assert MIRROR_TASK_DTYPE.itemsize == 48
TRANSPOSE_TASK_DTYPE = np.dtype([("in", np.uint64), ("out", np.uint64), ("rows", np.int64), ("cols", np.int64),
                                 ("tile_begin", np.int64)])
assert TRANSPOSE_TASK_DTYPE.itemsize == 40
ANTISYM_TASK_DTYPE = np.dtype([("rows", np.uint64), ("R", np.int64), ("N", np.int32), ("L", np.int32),
                               ("u", np.int32), ("mode", np.int32), ("nrow", np.int32), ("reserved", np.int32),
                               ("cta_begin", np.int64)])
assert ANTISYM_TASK_DTYPE.itemsize == 48
COEFF_TASK_DTYPE = np.dtype([("src", np.uint64), ("zT", np.uint64), ("zT32", np.uint64), ("n", np.int64),
                             ("K", np.int64), ("npad", np.int64), ("row_begin", np.int64)])
assert COEFF_TASK_DTYPE.itemsize == 56
ABT_TASK_DTYPE = np.dtype([("A", np.uint64), ("B", np.uint64), ("C", np.uint64), ("m", np.int64), ("n", np.int64),
                           ("K", np.int64), ("lda", np.int64), ("ldb", np.int64), ("alpha", np.float64),
                           ("cta_begin", np.int64), ("flags", np.int64)])
assert ABT_TASK_DTYPE.itemsize == 88
GEMV_TASK_DTYPE = np.dtype([("A", np.uint64), ("x", np.uint64), ("y", np.uint64), ("rows", np.int64),
                            ("cols", np.int64), ("lda", np.int64), ("alpha", np.float64), ("beta", np.float64),
                            ("row_begin", np.int64)])
assert GEMV_TASK_DTYPE.itemsize == 72
SPLIT_TASK_DTYPE = np.dtype([("src", np.uint64), ("hi", np.uint64), ("lo", np.uint64), ("rows", np.int64),
                             ("K", np.int64), ("ld", np.int64), ("Kp", np.int64), ("group_begin", np.int64)])
assert SPLIT_TASK_DTYPE.itemsize == 64
DENS_UNIT_DTYPE = np.dtype([("task", np.int32), ("idx", np.int32), ("c_lo", np.int32), ("c_hi", np.int32)])
assert DENS_UNIT_DTYPE.itemsize == 16
STATE_TASK_DTYPE = np.dtype([("gT", np.uint64), ("gT32", np.uint64), ("z", np.uint64), ("zn", np.uint64), ("G", np.uint64),
                             ("S", np.uint64), ("M", np.uint64), ("K", np.int64), ("n", np.int32),
                             ("reserved", np.int32), ("cta_begin", np.int64)])
assert STATE_TASK_DTYPE.itemsize == 80
SMALL_MM_TASK_DTYPE = np.dtype([("A", np.uint64), ("B", np.uint64), ("C", np.uint64), ("n", np.int32),
                                ("reserved", np.int32), ("alpha", np.float64), ("beta", np.float64),
                                ("cta_begin", np.int64)])
assert SMALL_MM_TASK_DTYPE.itemsize == 56
PERMUTE_TASK_DTYPE = np.dtype([("src", np.uint64), ("dst", np.uint64), ("dst_shape", np.int64, 6),
                               ("src_stride", np.int64, 6), ("ndim", np.int32), ("reserved", np.int32),
                               ("scale", np.float64), ("elem_begin", np.int64), ("n_elems", np.int64)])
assert PERMUTE_TASK_DTYPE.itemsize == 144
GATHER_TERMS_DTYPE = np.dtype([("src", np.uint64, 8), ("idx", np.uint64, 8), ("n_terms", np.int32),
                               ("reserved", np.int32)])
assert GATHER_TERMS_DTYPE.itemsize == 136
TASK_DTYPE = np.dtype([("M", np.int64), ("N", np.int64), ("seg_begin", np.int64), ("seg_count", np.int64),
                       ("mode", np.int64), ("splitk", np.int64), ("tile_begin", np.int64), ("C", np.uint64),
                       ("ldc", np.int64), ("rowA", np.uint64), ("colA", np.uint64), ("rowB", np.uint64),
                       ("colB", np.uint64), ("DA", np.uint64), ("DB", np.uint64), ("diagA", np.uint64),
                       ("diagB", np.uint64), ("batch", np.int64), ("sC", np.int64)])
assert SEGMENT_DTYPE.itemsize == 72 and TASK_DTYPE.itemsize == 152


class Transposes:
    """A fixed list of transposes (out = in^T for contiguous FP64 [rows, cols] inputs) run as
    one xrh_transpose_grouped launch."""

    def __init__(self, pairs, device):
        import torch
        tab = np.zeros(len(pairs), dtype=TRANSPOSE_TASK_DTYPE)
        tiles = 0
        for i, (src, dst, rows, cols) in enumerate(pairs):
            if src.dtype != torch.float64 or not src.is_contiguous() or not dst.is_contiguous():
                raise ValueError("grouped transposes need contiguous FP64 tensors")
            if src.numel() < rows * cols or dst.numel() < rows * cols:
                raise ValueError("transpose shape larger than its tensors")
            t = tab[i]
            t["in"], t["out"], t["rows"], t["cols"], t["tile_begin"] = src.data_ptr(), dst.data_ptr(), rows, cols, tiles
            tiles += ((rows + 31) // 32) * ((cols + 31) // 32)
        self.n, self.tiles = len(pairs), tiles
        self.keep = pairs
        self.dev = torch.from_numpy(tab.view(np.uint8).copy()).to(device) if len(pairs) else None

    def run(self, stream=None):
        if self.n:
            call("xrh_transpose_grouped", ptr(self.dev), self.n, self.tiles, stream_ptr(stream))


class Mirrors:
    """A fixed list of xrh_mirror_density calls [(src, dst, na, nb, N, L, accumulate)] run as
    one xrh_mirror_grouped launch (dst blocks distinct)."""

    def __init__(self, items, device):
        import torch
        dsts = [it[1].data_ptr() for it in items]
        if len(set(dsts)) != len(dsts):
            raise ValueError("grouped mirrors need distinct destination blocks")
        tab = np.zeros(len(items), dtype=MIRROR_TASK_DTYPE)
        cta = 0
        for i, (src, dst, na, nb, N, L, acc) in enumerate(items):
            if N > 64 or not 1 <= L <= 3:
                raise ValueError("mirror needs N <= 64 and 1 <= L <= 3")
            t = tab[i]
            t["src"], t["dst"], t["na"], t["nb"], t["N"], t["L"] = src.data_ptr(), dst.data_ptr(), na, nb, N, L
            t["accumulate"], t["cta_begin"] = int(acc), cta
            cta += na * nb * int(lib().xrh_mirror_ctas(N, L))
        self.n, self.ctas, self.keep = len(items), cta, items
        self.dev = torch.from_numpy(tab.view(np.uint8).copy()).to(device) if len(items) else None

    def run(self, stream=None):
        if self.n:
            call("xrh_mirror_grouped", ptr(self.dev), self.n, self.ctas, stream_ptr(stream))


class AntisymRows:
    """A fixed list of operator-pair row passes [(rows, R, N, L, u, mode)] run as one
    xrh_antisym_rows launch (the blocks distinct); modes 2 and 3 (Hermitian pairs) read the
    rows as square matrices (R a square)."""

    def __init__(self, items, device):
        import torch
        tab = np.zeros(len(items), dtype=ANTISYM_TASK_DTYPE)
        cta = 0
        for i, (rows, R, N, L, u, mode) in enumerate(items):
            nrow = int(round(R ** 0.5))
            if (not (0 <= u < L - 1) or mode not in (0, 1, 2, 3) or rows.numel() < (N ** L) * R or
                    (mode >= 2 and nrow * nrow != R)):
                raise ValueError("bad operator-pair row task")
            t = tab[i]
            t["rows"], t["R"], t["N"], t["L"], t["u"], t["mode"], t["cta_begin"] = rows.data_ptr(), R, N, L, u, mode, cta
            t["nrow"] = nrow if mode >= 2 else 0
            cta += N ** L
        self.n, self.ctas, self.keep = len(items), cta, items
        self.dev = torch.from_numpy(tab.view(np.uint8).copy()).to(device) if len(items) else None

    def run(self, stream=None):
        if self.n:
            call("xrh_antisym_rows", ptr(self.dev), self.n, self.ctas, stream_ptr(stream))


class PairLaunch:
    """A fixed list of pair scatters (gather=False: (pl, off, stride, zT, D, n)) or gathers
    (gather=True: (pl, off, stride, E, sigmaT, n)) run as one xrh_pair_grouped launch."""

    def __init__(self, items, gather, device):
        import torch
        tab = np.zeros(len(items), dtype=PAIR_TASK_DTYPE)
        mx = 0
        for i, (pl, off, stride, src, dst, n) in enumerate(items):
            t = tab[i]
            t["X"], t["xptr"] = pl["X_dev"].data_ptr(), pl["xptr_dev"].data_ptr()
            t["off"], t["sign"], t["stride"] = off.data_ptr(), pl["sign_dev"].data_ptr(), stride.data_ptr()
            t["src"], t["dst"], t["n"] = src.data_ptr(), dst.data_ptr(), n
            t["count"] = (pl["xptr_dev"].numel() - 1) if gather else len(pl["X"])
            mx = max(mx, int(t["count"]) * n)
        self.gather, self.n, self.max_total, self.keep = int(gather), len(items), mx, items
        self.dev = torch.from_numpy(tab.view(np.uint8).copy()).to(device) if len(items) else None

    def run(self, stream=None):
        if self.n:
            call("xrh_pair_grouped", self.gather, ptr(self.dev), self.n, self.max_total, stream_ptr(stream))


def zero_(t):
    """t[...] = 0 by cudaMemsetAsync on the current stream (no kernel; a memset node inside a
    captured graph)."""
    call("xrh_zero", ptr(t), t.numel() * t.element_size(), stream_ptr())
    return t

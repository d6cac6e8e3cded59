"""ctypes binding of the CUDA engine's C ABI (include/m25.h).

The shared library is built in-tree (mom25d_gb300/build.py). There is no
CPU fallback: loading fails loudly when the library or a CUDA device is
missing. Status codes map to the exceptions mom25d raises for the same
conditions (ValueError, MemoryError, RuntimeError).
"""

import atexit
import ctypes as C
import os
import sys
import weakref

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libm25.so")

M25_OK, M25_ERR_VALUE, M25_ERR_MEMORY, M25_ERR_CUDA, M25_ERR_NUMERIC = range(5)
M25_FP64, M25_MIXED, M25_MIXED_FILL32 = 0, 1, 2
M25_LU_NO_TENSOR_CORES = 1
M25_ON_HOST, M25_ON_DEVICE = 0, 1

EXPORTS = ("m25_last_error", "m25_version", "m25_ctx_create", "m25_ctx_destroy", "m25_ctx_synchronize",
           "m25_ctx_stream", "m25_geometry_create", "m25_geometry_destroy", "m25_geometry_stats",
           "m25_greens_create", "m25_greens_destroy", "m25_greens_tables", "m25_assemble", "m25_dense_solve",
           "m25_ports_create", "m25_ports_destroy", "m25_deembed", "m25_sweep_point", "m25_deembed_debug",
           "m25_ctx_timing", "m25_dense_solve_noalloc", "m25_lu_factor", "m25_greens_remainder", "m25_mlp_create",
           "m25_mlp_destroy", "m25_mlp_params", "m25_mlp_loss_grad", "m25_mlp_train", "m25_mlp_forward",
           "m25_ctx_mem_info", "m25_interp_create", "m25_interp_destroy", "m25_interp_store", "m25_interp_eval",
           "m25_interp_anchor", "m25_interp_point", "m25_deembed_waves", "m25_ctx_set_wait_limit",
           "m25_deembed_fit_info", "m25_ctx_set_tuning", "m25_ports_set_excitations", "m25_deembed_coefs",
           "m25_hmat_create", "m25_hmat_destroy", "m25_hmat_assemble", "m25_hmat_matvec", "m25_hmat_solve")

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)


class MeshDesc(C.Structure):
    _fields_ = [("nt", C.c_int32), ("nb", C.c_int32), ("nlev", C.c_int32),
                ("verts", _f64p), ("tri_basis", _i32p), ("tri_sign", _f64p), ("edge_len", _f64p),
                ("tri_layer", _i32p), ("level_z", _f64p), ("edge_tri", _i32p), ("edge_loc", _i32p),
                ("nblocks", C.c_int32), ("block_tris", _i32p),
                ("nv", C.c_int32), ("npad", C.c_int32), ("pad_tris", _i32p), ("seg_pad_off", _i32p),
                ("seg_pad", _i32p), ("seg_pad_w", _f64p), ("seg_end_lev", _i32p), ("seg_span", _f64p),
                ("seg_xy", _f64p), ("seg_drill", _f64p), ("near_factor", C.c_double), ("far_factor", C.c_double)]


class GreensDesc(C.Structure):
    _fields_ = [("freq", C.c_double), ("nlayer", C.c_int32), ("layer_t", _f64p), ("layer_eps", _f64p),
                ("layer_tand", _f64p), ("nlev", C.c_int32), ("lev_iface", _i32p), ("lev_z", _f64p),
                ("single", C.c_int32), ("zs_ground_re", C.c_double), ("zs_ground_im", C.c_double),
                ("stack_h", C.c_double), ("nk_c", C.c_int32), ("nk_r", C.c_int32), ("kc", _f64p), ("wc", _f64p),
                ("kr", _f64p), ("wr", _f64p), ("nrho", C.c_int32), ("rho", _f64p), ("kbig", C.c_double),
                ("surrogate", C.c_void_p), ("sur_a", C.c_double), ("sur_rho_ref", C.c_double),
                ("sur_fmin", C.c_double), ("sur_fmax", C.c_double), ("sur_scale", _f64p), ("sur_near", C.c_double),
                ("sur_stride", C.c_int32), ("sur_tol", C.c_double), ("top_pec", C.c_int32)]


class PortDesc(C.Structure):
    _fields_ = [("nport", C.c_int32), ("ngroup", C.c_int32), ("group_of", _i32p), ("port_level", _i32p),
                ("ns", _i32p), ("s", _f64p), ("cut_off", _i32p), ("cut_edge", _i32p), ("cut_w", _f64p),
                ("nvpt", _i32p), ("vpts", _f64p), ("beta0", _f64p), ("lossless", C.c_int32), ("bounds", _f64p),
                ("v_weight", C.c_double), ("excitation", _f64p)]


_i64p = C.POINTER(C.c_int64)


class HmatDesc(C.Structure):
    _fields_ = [("nb", C.c_int32), ("nv", C.c_int32), ("perm", _i32p), ("rules", _f64p), ("lev", _i32p),
                ("nleaf", C.c_int32), ("leaf_lo", _i32p), ("nnear", C.c_int32), ("near", _i32p),
                ("nfar", C.c_int32), ("far", _i32p), ("far_cen", _i32p), ("ent_off", _i64p), ("ent", _i32p),
                ("nkeys", C.c_int64), ("keys", _i64p), ("npblk", C.c_int32), ("pblk", _i32p), ("npc", C.c_int32),
                ("pc_off", _i64p), ("pc_gidx", _i32p), ("pc_own", C.POINTER(C.c_int8)), ("pc_item_off", _i64p),
                ("pc_items", _i32p), ("tol", C.c_double), ("kcap", C.c_int32)]


_lib = None


def load():
    """The engine library (built on demand when nvcc is present)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build

        build.build()
    lib = C.CDLL(LIB_PATH)
    for name in EXPORTS:
        getattr(lib, name)  # every declared entry point must be exported
    lib.m25_last_error.restype = C.c_char_p
    lib.m25_ctx_stream.restype = C.c_void_p
    vp = C.c_void_p
    lib.m25_ctx_create.argtypes = [C.c_int, C.POINTER(vp)]
    for f in ("m25_ctx_destroy", "m25_ctx_synchronize", "m25_geometry_destroy", "m25_greens_destroy",
              "m25_ports_destroy"):
        getattr(lib, f).argtypes = [vp]
    lib.m25_geometry_create.argtypes = [vp, C.POINTER(MeshDesc), C.POINTER(vp)]
    lib.m25_geometry_stats.argtypes = [vp, C.POINTER(C.c_int64)]
    lib.m25_greens_create.argtypes = [vp, C.POINTER(GreensDesc), C.POINTER(vp)]
    lib.m25_greens_tables.argtypes = [vp, _f64p, _f64p, _f64p]
    d = C.c_double
    lib.m25_assemble.argtypes = [vp, vp, vp, d, d, d, d, C.c_int, vp, C.c_int64, C.c_int]
    lib.m25_dense_solve.argtypes = [vp, C.c_int32, C.c_int32, C.c_int, vp, vp, vp, C.c_int, d, C.c_int32, _i32p]
    lib.m25_ports_create.argtypes = [vp, vp, C.POINTER(PortDesc), C.POINTER(vp)]
    lib.m25_deembed.argtypes = [vp, vp, vp, vp, vp, C.c_int, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p]
    lib.m25_sweep_point.argtypes = [vp, vp, vp, vp, d, d, d, d, C.c_int, _f64p, d, C.c_int32, _f64p, _f64p, _f64p,
                                    _f64p, _f64p, _f64p, _i32p]
    lib.m25_deembed_debug.argtypes = [vp, vp, _f64p, _f64p, _f64p, _f64p]
    lib.m25_deembed_waves.argtypes = [vp, _f64p]
    lib.m25_deembed_fit_info.argtypes = [vp, _i32p]
    lib.m25_ports_set_excitations.argtypes = [vp, C.c_int32]
    lib.m25_deembed_coefs.argtypes = [vp, _f64p, _f64p]
    lib.m25_ctx_timing.argtypes = [vp, C.c_int, _f64p, C.POINTER(C.c_longlong)]
    lib.m25_dense_solve_noalloc.argtypes = [C.c_int32, C.c_int32, vp, vp, vp, vp, vp, _i32p]
    lib.m25_lu_factor.argtypes = [vp, C.c_int32, C.c_int, vp, C.c_int64, _i32p, C.c_int, C.c_int32, _i32p]
    lib.m25_greens_remainder.argtypes = [vp, _f64p, _f64p]
    lib.m25_ctx_mem_info.argtypes = [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    lib.m25_ctx_set_wait_limit.argtypes = [vp, C.c_int64]
    lib.m25_ctx_set_tuning.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    lib.m25_interp_create.argtypes = [vp, C.c_int32, C.c_int32, _f64p, C.c_int32, C.c_int32, C.POINTER(vp)]
    lib.m25_interp_destroy.argtypes = [vp]
    lib.m25_interp_store.argtypes = [vp, C.c_int32, vp, C.c_int64, C.c_int, d, d]
    lib.m25_interp_eval.argtypes = [vp, C.c_int32, _i32p, _f64p, d, d, vp, C.c_int64, C.c_int]
    lib.m25_interp_anchor.argtypes = [vp, vp, vp, vp, C.c_int32, d, d, d, d, C.c_int, d]
    lib.m25_interp_point.argtypes = [vp, vp, vp, vp, vp, C.c_int32, _i32p, _f64p, d, C.c_int, _f64p, d, C.c_int32,
                                     _f64p, _f64p, _f64p, _f64p, _f64p, _f64p, _i32p]
    lib.m25_hmat_create.argtypes = [vp, vp, C.POINTER(HmatDesc), C.POINTER(vp)]
    lib.m25_hmat_destroy.argtypes = [vp]
    lib.m25_hmat_assemble.argtypes = [vp, vp, d, d, d, d, _i64p]
    lib.m25_hmat_matvec.argtypes = [vp, _f64p, _f64p]
    lib.m25_hmat_solve.argtypes = [vp, C.c_int32, _f64p, _f64p, d, C.c_int32, C.c_int32, _i32p, _f64p]
    f32p = C.POINTER(C.c_float)
    lib.m25_mlp_create.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.POINTER(vp)]
    lib.m25_mlp_destroy.argtypes = [vp]
    lib.m25_mlp_params.argtypes = [vp, C.POINTER(C.c_int64), f32p, f32p]
    lib.m25_mlp_loss_grad.argtypes = [vp, C.c_int32, f32p, f32p, _f64p, f32p]
    lib.m25_mlp_train.argtypes = [vp, C.c_int32, f32p, f32p, C.c_int32, C.c_int32, d, d, C.c_uint64, _f64p]
    lib.m25_mlp_forward.argtypes = [vp, C.c_int32, f32p, f32p]
    _lib = lib
    return lib


class NumericError(RuntimeError):
    """M25_ERR_NUMERIC: a zero pivot, or a refinement that stopped above its
    target (a RuntimeError, as mom25d raises for a failed iterative solve)."""


def check(rc):
    if rc == M25_OK:
        return
    msg = load().m25_last_error().decode(errors="replace")
    if rc == M25_ERR_VALUE:
        raise ValueError(msg)
    if rc == M25_ERR_MEMORY:
        raise MemoryError(msg)
    if rc == M25_ERR_NUMERIC:
        raise NumericError(msg)
    raise RuntimeError(msg)


def ptr(a, ctype=C.c_double):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None else None


def i32(a):
    return np.ascontiguousarray(a, np.int32)


def f64(a):
    return np.ascontiguousarray(a, np.float64)


_live_contexts = weakref.WeakSet()


class Context:
    """One engine context: a CUDA device and stream plus a reusable workspace.
    Device objects created in it (Handle) are released before it."""

    def __init__(self, device=0):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.m25_ctx_create(int(device), C.byref(h)))
        self.h = h
        self.device = device
        self.handles = weakref.WeakSet()
        _live_contexts.add(self)

    def close(self):
        if getattr(self, "h", None):
            for hd in list(self.handles):
                hd.close()
            self.lib.m25_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def synchronize(self):
        check(self.lib.m25_ctx_synchronize(self.h))


@atexit.register
def _close_all():
    # before the CUDA runtime's own teardown
    for c in list(_live_contexts):
        try:
            c.close()
        except Exception:  # noqa: BLE001
            pass


class Handle:
    """Owner of a device object (geometry, Green's tables, ports) of a Context."""

    def __init__(self, ctx, h, destroy):
        self.ctx, self.h, self._destroy = ctx, h, destroy
        ctx.handles.add(self)

    def close(self):
        if self.h and self.ctx.h:
            self._destroy(self.h)
        self.h = None

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

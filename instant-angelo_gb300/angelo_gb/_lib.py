"""ctypes binding of libangelo_gb.so (the C ABI declared in include/angelo_gb.h).

The library is the only compute path: if it is missing or does not load, every
op raises instead of falling back to anything else."""
from __future__ import annotations

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libangelo_gb.so")

ANGELO_OK = 0
ANGELO_E_INVALID = 1
ANGELO_E_CUDA = 2
ANGELO_E_UNSUPPORTED = 3
ANGELO_E_CAPACITY = 4
MAX_LEVELS = 32
DTYPE_F32 = 0
DTYPE_F16 = 1
OPERAND_BF16 = 0
OPERAND_FP16 = 1

c_i32, c_i64, c_f32, c_vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p


class HashGridDesc(ctypes.Structure):
    _fields_ = [("n_levels", c_i32), ("n_features", c_i32), ("log2_hashmap_size", c_i32),
                ("base_resolution", c_i32), ("per_level_scale", c_f32)]


class HashGridLayout(ctypes.Structure):
    _fields_ = [("n_levels", c_i32), ("n_features", c_i32),
                ("offsets", ctypes.c_uint32 * (MAX_LEVELS + 1)),
                ("resolutions", ctypes.c_uint32 * MAX_LEVELS),
                ("scales", c_f32 * MAX_LEVELS)]


class GridDesc(ctypes.Structure):
    _fields_ = [("roi", c_f32 * 6), ("res", c_i32 * 3), ("bits", c_vp), ("contraction", c_i32)]


CONTRACT_AABB, CONTRACT_UNBOUNDED_SPHERE = 0, 1


class SdfNetLayout(ctypes.Structure):
    _fields_ = [("k_tiles1", c_i32), ("n_hidden", c_i32), ("n_tiles3", c_i32),
                ("k_tiles3b", c_i32), ("out_dim", c_i32),
                ("off_b1", c_i64), ("off_b2", c_i64), ("off_b3", c_i64),
                ("off_w3row0", c_i64), ("off_tcw1", c_i64), ("off_tcw2", c_i64),
                ("off_tcw3", c_i64), ("bytes", c_i64), ("mma_passes", c_i32),
                ("operand_format", c_i32)]


class ServeField(ctypes.Structure):
    _fields_ = [("lay", HashGridLayout), ("active_levels", c_i32), ("table", c_vp),
                ("table_dtype", c_i32), ("sdf_layout", SdfNetLayout), ("sdf_net", c_vp),
                ("radius", c_f32), ("eps", c_f32), ("feat_dim", c_i32), ("rad_net", c_vp),
                ("rad_flags", c_i32), ("variance", c_vp), ("cos_anneal_ratio", c_f32),
                ("background", c_vp), ("grid", GridDesc), ("render_step", c_f32),
                ("max_steps", c_i32), ("near_plane", c_f32), ("far_plane", c_f32)]


class AngeloError(RuntimeError):
    def __init__(self, fn, code, msg):
        super().__init__(f"{fn} failed with status {code}: {msg}")
        self.code = code


# name -> (restype, argtypes)
_P = ctypes.POINTER
SIGNATURES = {
    "angelo_last_error_string": (ctypes.c_char_p, []),
    "angelo_version": (c_i32, []),
    "angelo_hashgrid_layout": (c_i32, [_P(HashGridDesc), _P(HashGridLayout)]),
    "angelo_hashgrid_fwd": (c_i32, [_P(HashGridLayout), c_i32, c_vp, c_i64, c_vp, c_i32, c_i32,
                                    c_vp, c_i64, c_i64, c_vp]),
    "angelo_hashgrid_bwd": (c_i32, [_P(HashGridLayout), c_i32, c_vp, c_i64, c_vp, c_i32, c_i32,
                                    c_vp, c_i64, c_i64, c_vp, c_vp, c_vp]),
    "angelo_hashgrid_index": (c_i32, [_P(HashGridLayout), c_vp, c_i64, c_vp, c_vp, c_vp]),
    "angelo_sh4_fwd": (c_i32, [c_vp, c_i64, c_i32, c_vp, c_i64, c_i64, c_vp]),
    "angelo_sh4_bwd": (c_i32, [c_vp, c_i64, c_i32, c_vp, c_i64, c_i64, c_vp, c_vp]),
    "angelo_ray_aabb": (c_i32, [c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp]),
    "angelo_march_count": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_i64, _P(GridDesc), c_f32, c_f32,
                                   c_i64, c_vp, c_vp, c_vp]),
    "angelo_scan_workspace_size": (c_i64, [c_i64]),
    "angelo_scan": (c_i32, [c_vp, c_i64, c_vp, c_vp, c_vp]),
    "angelo_scan_noalloc": (c_i32, [c_vp, c_i64, c_vp, c_vp]),
    "angelo_march_fill": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_i64, _P(GridDesc), c_f32, c_f32,
                                  c_i64, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "angelo_offsets_clamp": (c_i32, [c_vp, c_i64, c_i64, c_vp]),
    "angelo_march_record": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_i64, _P(GridDesc), c_f32, c_f32,
                                    c_i64, c_i32, c_vp, c_vp, c_vp, c_vp]),
    "angelo_march_compact": (c_i32, [c_vp, c_i32, c_vp, c_vp, c_i64, c_i64, c_vp, c_vp, c_vp, c_vp,
                                     c_vp]),
    "angelo_occ_workspace_size": (c_i64, [c_i64]),
    "angelo_occ_update": (c_i32, [c_vp, c_i64, c_vp, c_vp, c_i64, c_f32, c_f32, c_vp, c_vp,
                                  c_vp]),
    "angelo_density_weights_fwd": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp]),
    "angelo_density_weights_bwd": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp]),
    "angelo_mc_workspace_size": (c_i64, [c_i32, c_i32, c_i32]),
    "angelo_mc_count": (c_i32, [c_vp, c_i32, c_i32, c_i32, c_f32, c_vp, c_vp, c_vp]),
    "angelo_mc_extract": (c_i32, [c_vp, c_i32, c_i32, c_i32, c_f32, c_vp, c_vp, c_vp, c_vp, c_vp,
                                  c_vp]),
    "angelo_weights_fwd": (c_i32, [c_vp, c_vp, c_i64, c_f32, c_vp, c_vp, c_vp]),
    "angelo_weights_bwd": (c_i32, [c_vp, c_vp, c_vp, c_i64, c_f32, c_vp, c_vp, c_vp]),
    "angelo_accumulate_fwd": (c_i32, [c_vp, c_vp, c_i32, c_vp, c_i64, c_vp, c_vp]),
    "angelo_accumulate_bwd": (c_i32, [c_vp, c_vp, c_i32, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp]),
    "angelo_sdf_net_layout_query": (c_i32, [c_i32, c_i32, c_i32, _P(SdfNetLayout)]),
    "angelo_sdf_prep": (c_i32, [_P(SdfNetLayout), c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp,
                                c_vp, c_vp, c_vp]),
    "angelo_sdf_grad_size": (c_i64, [_P(SdfNetLayout)]),
    "angelo_sdf_workspace_floats": (c_i64, [_P(HashGridLayout), c_i64, c_i32, c_i32, c_i32]),
    "angelo_sdf_stencil_fwd": (c_i32, [_P(HashGridLayout), c_i32, c_vp, c_i32, _P(SdfNetLayout),
                                       c_vp, c_vp, c_vp, c_i64, c_f32, c_f32, c_i32, c_i32, c_i32,
                                       c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp]),
    "angelo_sdf_stencil_bwd": (c_i32, [_P(HashGridLayout), c_i32, c_vp, c_i32, _P(SdfNetLayout),
                                       c_vp, c_vp, c_vp, c_i64, c_f32, c_f32, c_i32, c_i32, c_vp,
                                       c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp]),
    "angelo_tc_timeouts": (c_i64, [c_i32]),
    "angelo_adamw_step": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_i64, c_f32, c_f32, c_f32, c_f32, c_f32,
                                  c_f32, c_f32, c_vp]),
    "angelo_adamw_step_multi": (c_i32, [c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                        c_vp, c_vp, c_vp, c_vp]),
    "angelo_weight_norm_fwd": (c_i32, [c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "angelo_weight_norm_bwd": (c_i32, [c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "angelo_loss_workspace_size": (c_i64, []),
    "angelo_neus_loss_fwd": (c_i32, [c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_i64, c_f32, c_f32, c_f32,
                                     c_vp, c_vp, c_vp]),
    "angelo_neus_loss_bwd": (c_i32, [c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_i64, c_f32, c_f32, c_f32,
                                     c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "angelo_radiance_net_bytes": (c_i64, [c_i32]),
    "angelo_radiance_grad_size": (c_i64, [c_i32]),
    "angelo_radiance_prep": (c_i32, [c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "angelo_radiance_prep_format": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                            c_vp]),
    "angelo_radiance_fwd": (c_i32, [c_i32, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_i64, c_i32, c_vp,
                                    c_vp]),
    "angelo_radiance_bwd": (c_i32, [c_i32, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_i64, c_i32, c_vp,
                                    c_vp, c_vp, c_vp, c_vp]),
    "angelo_mlp_net_bytes": (c_i64, [c_i32, c_i32, c_i32]),
    "angelo_mlp_grad_size": (c_i64, [c_i32, c_i32, c_i32]),
    "angelo_mlp_prep": (c_i32, [c_i32, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "angelo_mlp_fused_fwd": (c_i32, [c_i32, c_i32, c_i32, c_vp, c_vp, c_i64, c_i64, c_vp, c_i64, c_vp]),
    "angelo_mlp_fused_bwd": (c_i32, [c_i32, c_i32, c_i32, c_vp, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64,
                                     c_vp, c_i64, c_vp, c_vp]),
    "angelo_density_composite_fwd": (c_i32, [c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                             c_vp, c_vp, c_vp, c_vp]),
    "angelo_density_composite_bwd": (c_i32, [c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                             c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "angelo_sample_points": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp]),
    "angelo_bg_points": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_f32, c_vp, c_vp]),
    "angelo_bg_visibility": (c_i32, [c_vp, c_i64, c_f32, c_vp, c_vp, c_vp, c_i64, c_f32, c_vp, c_vp]),
    "angelo_bg_compact": (c_i32, [c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp,
                                  c_vp, c_vp, c_vp, c_vp, c_vp]),
    "angelo_serve_field_bytes": (c_i64, []),
    "angelo_serve_create": (c_i32, [c_vp, c_i64, c_i32, c_i64, c_i32, c_vp]),
    "angelo_serve_render": (c_i32, [c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "angelo_serve_sdf": (c_i32, [c_vp, c_vp, c_i64, c_vp, c_vp]),
    "angelo_serve_destroy": (c_i32, [c_vp]),
    "angelo_composite_fwd": (c_i32, [c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_f32,
                                     c_vp, c_f32, c_f32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                     c_vp, c_vp, c_vp]),
    "angelo_composite_bwd": (c_i32, [c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_f32,
                                     c_vp, c_f32, c_f32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                     c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
}

_lock = threading.Lock()
_lib = None


def load(path: str = None):
    """Load libangelo_gb.so and bind every entry point of the C ABI.  The
    library next to this package, or the file $ANGELO_GB_LIB names (a build
    of the same sources with other compile-time settings)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or os.environ.get("ANGELO_GB_LIB") or LIB_PATH
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise RuntimeError(
                    f"libangelo_gb.so not found at {path}: build it with "
                    "`python -m angelo_gb.build` (needs nvcc); there is no fallback path")
            L = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


class Profiler:
    """Opt-in record of library calls: CUDA events on the launching stream
    around each call, the kernel launches it made and its work units.  Used
    by bench.py to time the dominant kernel inside the timed region."""

    def __init__(self):
        self.active = False
        self.records = []      # (name, start_event, end_event, units)
        self.launches = 0

    def start(self):
        self.records, self.launches, self.active = [], 0, True

    def stop(self):
        self.active = False

    def summary(self):
        """{name: (calls, total_ms, [units...])} after synchronisation."""
        out = {}
        for name, s, e, units in self.records:
            c, t, u = out.get(name, (0, 0.0, []))
            u.append(units)
            out[name] = (c + 1, t + s.elapsed_time(e), u)
        return out


PROFILER = Profiler()


def call(name, *args, launches=1, units=None, stream=None):
    """Call an int-status entry point; raise AngeloError on a non-zero status.
    ``launches`` is the number of kernels the call puts on the stream and
    ``units`` its work description, both only recorded while profiling."""
    L = load()
    if name not in SIGNATURES:
        # a function without declared argument types would receive Python
        # ints as 32-bit C ints: refuse instead of launching with garbage
        raise AngeloError(name, ANGELO_E_INVALID, "entry point has no registered signature")
    prof = PROFILER.active
    if prof:
        import torch
        s = torch.cuda.current_stream()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(s)
    rc = getattr(L, name)(*args)
    if rc != ANGELO_OK:
        msg = L.angelo_last_error_string().decode(errors="replace")
        raise AngeloError(name, rc, msg)
    if prof:
        ev1.record(s)
        PROFILER.records.append((name, ev0, ev1, units))
        PROFILER.launches += launches
    return rc


def raw(name):
    return getattr(load(), name)

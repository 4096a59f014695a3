"""ctypes binding of libmeshode.so (declared in include/meshode.h).

The library is the only compute path: importing an entry point when the
shared object is missing, or when no CUDA device is present, raises.
"""
import ctypes
import os

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmeshode.so")

MO_OK, MO_ERR_INVALID, MO_ERR_CUDA, MO_ERR_SCRATCH, MO_ERR_DEVICE = 0, 1, 2, 3, 4
MO_LAYOUT_LINEAR, MO_LAYOUT_CELL, MO_LAYOUT_BRICK4 = 0, 1, 2
MO_PACKET_4x4x2, MO_PACKET_8x4x1, MO_PACKET_4x2x4, MO_PACKET_2x4x4, MO_PACKET_8x2x2 = 0, 1, 2, 3, 4
MO_PACKET_4x4x4, MO_PACKET_2x4x8, MO_PACKET_8x4x2 = 5, 6, 7
MO_PACKET_4x4x2_TRI2, MO_PACKET_2x4x4_TRI2 = 8, 9
MO_DF_AUTO, MO_DF_BRUTE, MO_DF_LBVH = 0, 1, 2
MO_EDGES_FACES, MO_EDGES_LIST = 0, 1
MO_TILE_WARPS = 8
MO_REQ_FAILED, MO_REQ_QUEUED, MO_REQ_BUILDING, MO_REQ_ACTIVE, MO_REQ_DONE = -1, 0, 1, 2, 3
MO_DF_FULL, MO_DF_ON_DEMAND = 0, 1
MO_DF_LAZY_MAX_N = 1024

_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_F = ctypes.c_float
_SZ = ctypes.c_size_t


class MoPair(ctypes.Structure):
    _fields_ = [
        ("grid", _P), ("slice_ptr", _P), ("sell", _P), ("rest", _P), ("pos0", _P), ("pos1", _P),
        ("adam_m", _P), ("adam_v", _P), ("adam_tab", _P), ("grad_dbg", _P),
        ("N", ctypes.c_int32), ("layout", ctypes.c_int32), ("nv", ctypes.c_int32), ("nslices", ctypes.c_int32),
        ("w_edge", _F), ("mask_thresh", _F), ("use_mask", ctypes.c_int32), ("grad_scale", _F),
        ("one_minus_b1", _F), ("b2", _F), ("one_minus_b2", _F), ("eps", _F),
        ("t0", ctypes.c_int32), ("t_end", ctypes.c_int32), ("tile0", ctypes.c_int32), ("ntiles", ctypes.c_int32),
        ("df_tree", _P), ("df_lin", _P), ("df_cells", _P), ("df_packets", _P), ("df_status", _P),
        ("df_queue", _P), ("df_pqueue", _P), ("df_queue_count", _P), ("df_ntri", ctypes.c_int32), ("df_queue_cap", ctypes.c_int32),
        ("df_band", _F), ("df_pad", ctypes.c_int32), ("sell_w", _P),
    ]


class MoDfOptions(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int32), ("packet", ctypes.c_int32), ("band", _F), ("reserved", ctypes.c_int32)]


class MoTile(ctypes.Structure):
    _fields_ = [("pair", ctypes.c_int32), ("slice0", ctypes.c_int32), ("nslices", ctypes.c_int32),
                ("pad", ctypes.c_int32)]


class MoPoolConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_pairs", ctypes.c_int32),
                ("max_tiles", ctypes.c_int32), ("group_steps", ctypes.c_int32), ("use_graph", ctypes.c_int32),
                ("max_building", ctypes.c_int32), ("build_streams", ctypes.c_int32), ("layout", ctypes.c_int32),
                ("slices_per_tile", ctypes.c_int32), ("step_grid", ctypes.c_int32), ("df_mode", ctypes.c_int32)]


class MoRequest(ctypes.Structure):
    _fields_ = [("srcV", _P), ("srcF", _P), ("tarV", _P), ("tarF", _P),
                ("nv", _I64), ("nf", _I64), ("ntv", _I64), ("ntf", _I64),
                ("inputs_on_host", ctypes.c_int32), ("N", ctypes.c_int32), ("steps", ctypes.c_int32),
                ("w_edge", _F), ("lr", ctypes.c_double), ("layout", ctypes.c_int32),
                ("slices_per_tile", ctypes.c_int32), ("df_method", ctypes.c_int32), ("df_packet", ctypes.c_int32),
                ("df_band", _F), ("out_on_host", ctypes.c_int32), ("V_out", _P), ("V_normalized_out", _P)]


class MoPoolStats(ctypes.Structure):
    _fields_ = [("submitted", _I64), ("done", _I64), ("failed", _I64), ("groups", _I64),
                ("fused_launches", _I64), ("bytes_in_use", ctypes.c_uint64), ("peak_bytes", ctypes.c_uint64),
                ("queued", ctypes.c_int32), ("building", ctypes.c_int32), ("active", ctypes.c_int32),
                ("retiring", ctypes.c_int32), ("active_tiles", ctypes.c_int32),
                ("fill_launches_per_step", ctypes.c_int32)]


# name -> (restype, argtypes)
_SIGS = {
    "mo_last_error": (ctypes.c_char_p, []),
    "mo_version": (_I, []),
    "mo_launch_count": (ctypes.c_ulonglong, []),
    "mo_bbox": (_I, [_P, _I64, _P, _P]),
    "mo_norm_params": (_I, [_P, _P, _P]),
    "mo_normalize": (_I, [_P, _I64, _P, _I, _P]),
    "mo_df_build_scratch_bytes": (_SZ, [_I64, _I64, _I, _I]),
    "mo_df_build": (_I, [_P, _I64, _P, _I64, _I, _P, _I, _P, _SZ, _P, _P, _P]),
    "mo_df_method_for": (_I, [_I64, _I]),
    "mo_df_loss_band": (_F, [_I]),
    "mo_df_build_ex": (_I, [_P, _I64, _P, _I64, _I, _P, _P, _P, _SZ, _P, _P, _P]),
    "mo_df_build_count": (_I, [_P, _I64, _P, _I64, _I, _P, _P, _P, _SZ, _P, _P, _P, _P]),
    "mo_df_build_noalloc": (_I, [_P, _I64, _P, _I64, _I, _P, _P, _P]),
    "mo_df_noalloc_scratch_capacity": (_SZ, []),
    "mo_df_tree_bytes": (_SZ, [_I64]),
    "mo_df_tree_scratch_bytes": (_SZ, [_I64, _I64]),
    "mo_df_tree_build": (_I, [_P, _I64, _P, _I64, _P, _P, _SZ, _P, _P, _P]),
    "mo_df_lazy_bytes": (_SZ, [_I]),
    "mo_df_lazy_seed": (_I, [_P, _I, _P, _I64, _P, _P, _P, _I, _P]),
    "mo_df_lazy_fill": (_I, [_P, _P, _P, _P, _I, _P, _P]),
    "mo_lbvh_build": (_I, [_P, _I64, _P, _I64, _P, _P, _SZ, _P, _P, _P, _P, _P, _P]),
    "mo_grid_bytes": (_SZ, [_I, _I]),
    "mo_grid_relayout": (_I, [_P, _I, _I, _P, _P]),
    "mo_dfloss_forward": (_I, [_P, _I64, _P, _I, _I, _P, _P]),
    "mo_dfloss_backward": (_I, [_P, _I64, _P, _I, _I, _P, _P]),
    "mo_dfloss_fwd_bwd": (_I, [_P, _I64, _P, _I, _I, _P, _P, _I, _F, _P]),
    "mo_edge_count": (_I64, [_I64, _I]),
    "mo_edge_offsets": (_I, [_P, _I64, _P, _I64, _I, _P, _P]),
    "mo_edge_forward": (_I, [_P, _I64, _P, _I64, _I, _P, _P, _P]),
    "mo_edge_csr_bytes": (_SZ, [_I64, _I64, _I]),
    "mo_edge_csr_build": (_I, [_P, _I64, _I, _I64, _P, _SZ, _P, _P]),
    "mo_edge_backward": (_I, [_P, _I64, _P, _I64, _P, _P, _P]),
    "mo_edge_cad_list": (_I, [_P, _I64, _P, _I64, _P, _P]),
    "mo_edge_cad_weights": (_I, [_P, _I64, _P, _P]),
    "mo_edge_forward_w": (_I, [_P, _I64, _P, _I64, _I, _P, _P, _P, _P]),
    "mo_edge_backward_w": (_I, [_P, _I64, _P, _I64, _P, _P, _P, _P]),
    "mo_edge_fwd_bwd": (_I, [_P, _I64, _P, _I64, _I, _P, _P, _P, _P, _P, _P]),
    "mo_sell_plan": (_I, [_P, _I64, _I64, _P, _P]),
    "mo_sell_fill": (_I, [_P, _I64, _I64, _P, _P, _P]),
    "mo_sell_fill_w": (_I, [_P, _I64, _I64, _P, _P, _P, _P]),
    "mo_adam_step": (_I, [_P, _P, _P, _P, _I64, _F, _F, _F, _F, _F, _F, _P]),
    "mo_fused_step": (_I, [_P, _P, _P, _I, _I, _P, _I, _P]),
    "mo_fused_step_weighted": (_I, [_P, _P, _P, _I, _I, _P, _I, _P]),
    "mo_fused_step_on_demand": (_I, [_P, _P, _P, _I, _I, _P, _I, _P]),
    "mo_pair_loss": (_I, [_P, _I, _I, _I, _P, _P, _P]),
    "mo_abi_sizes": (_I, [ctypes.POINTER(_SZ), ctypes.POINTER(_SZ)]),
    "mo_mlp_width": (_I, []),
    "mo_mlp_tiles": (_I64, [_I64]),
    "mo_mlp_partial_floats": (_I, []),
    "mo_mlp_transpose": (_I, [_P, _P, _P]),
    "mo_mlp_fwd": (_I, [_P, _P, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _F, _F, _I, _P, _P, _P, _I64, _P]),
    "mo_mlp_bwd": (_I, [_P, _P, _I64, _P, _P, _P, _P, _P, _I64, _P, _P, _P, _P, _P]),
    "mo_mlp_partial_reduce_bytes": (_SZ, []),
    "mo_mlp_partial_reduce": (_I, [_P, _I64, _P, _P, _P, _P, _P, _P, _P, _P]),
    "mo_mlp_wgrad_partial_bytes": (_SZ, [_I]),
    "mo_mlp_wgrad": (_I, [_P, _P, _I64, _I, _P, _P, _P]),
    "mo_pack_pos": (_I, [_P, _I64, _P, _P]),
    "mo_unpack_pos": (_I, [_P, _I64, _P, _P]),
    "mo_nn_scratch_bytes": (_SZ, [_I64, _I64]),
    "mo_nn_query": (_I, [_P, _I64, _P, _I64, _P, _P, _P, _SZ, _P]),
    "mo_reverse_loss_scratch_bytes": (_SZ, [_I64, _I64]),
    "mo_reverse_loss_forward": (_I, [_P, _I64, _P, _I64, _P, _P, _P, _SZ, _P, _P]),
    "mo_reverse_loss_backward": (_I, [_P, _I64, _P, _I64, _P, _P, _P, _P, _SZ, _P, _P]),
    "mo_solve_linear_scratch_bytes": (_SZ, [_I64, _I64, _I64, _I64, _I]),
    "mo_solve_linear": (_I, [_P, _I64, _P, _I64, _P, _I64, _P, _P, _I64, ctypes.c_double, _I, ctypes.c_double, _I,
                             _P, _SZ, _P, _P, _P]),
    "mo_pool_create": (_I, [_P, _P]),
    "mo_pool_destroy": (_I, [_P]),
    "mo_pool_submit": (_I, [_P, _P, _P]),
    "mo_pool_progress": (_I, [_P, _I, _P]),
    "mo_pool_wait": (_I, [_P]),
    "mo_pool_completed": (_I, [_P, _P, _I, _P]),
    "mo_pool_state": (_I, [_P, _I64, _P]),
    "mo_pool_error": (_I, [_P, _I64, _P, _SZ]),
    "mo_pool_result": (_I, [_P, _I64, _P, _P, _I, _P]),
    "mo_pool_release": (_I, [_P, _I64]),
    "mo_pool_set_hold": (_I, [_P, _I]),
    "mo_pool_set_timing": (_I, [_P, _I]),
    "mo_pool_run_groups": (_I, [_P, _I]),
    "mo_pool_group_time": (_I, [_P, _P, _P]),
    "mo_pool_stats": (_I, [_P, _P]),
    "mo_pool_fill_totals": (_I, [_P, _P]),
    "mo_pool_trim": (_I, [_P, ctypes.c_uint64]),
    "mo_pool_step_stream": (_I, [_P, _P]),
}

_lib = None


class MeshodeError(RuntimeError):
    pass


def lib():
    """Load libmeshode.so once; raise if it is missing (no CPU fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise MeshodeError(
                "libmeshode.so is not built (%s); run `python -c \"import __graft_entry__ as g; g.build()\"`"
                % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return sorted(_SIGS)


def check(rc, what=""):
    if rc != MO_OK:
        msg = lib().mo_last_error()
        msg = msg.decode() if msg else ""
        raise MeshodeError("%s failed (status %d): %s" % (what, rc, msg))


def call(name, *args):
    """Call an entry point and raise MeshodeError on a non-zero status."""
    rc = getattr(lib(), name)(*args)
    check(rc, name)
    return rc


def require_cuda():
    if not torch.cuda.is_available():
        raise MeshodeError("meshode_gb300 needs a CUDA device (GB300 / sm_103a); none is available")
    lib()


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)

"""ctypes binding of libffsrl_cuda.so (declarations in include/ffsrl.h).

The library is required: importing the product modules without it built raises
``FFSRLError`` rather than falling back to any other implementation.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "libffsrl_cuda.so"

# status codes (ffsrl_status)
OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_CUDA = 2
ERR_OUT_OF_MEMORY = 3
ERR_BUDGET = 4
ERR_TIMEOUT = 5
ERR_UNSUPPORTED = 6
ERR_NONFINITE = 7
ERR_STACK_OVERFLOW = 8
ERR_BUSY = 9
ERR_NOT_FOUND = 10

# ffsrl_params.flags
VOLUME = 1 << 0
DISTANCE = 1 << 1
NEOHOOKEAN = 1 << 2
DISTANCE_XPBD = 1 << 3
VOLUME_XPBD = 1 << 4
DRAG = 1 << 5
CONNECTORS = 1 << 6
COLLIDE = 1 << 7
REFERENCE_STEP = VOLUME | DISTANCE | DRAG | CONNECTORS | COLLIDE


class FFSRLError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ffsrl error {code}: {msg}")
        self.code = code


P = C.c_void_p
I32 = C.c_int32
F32 = C.c_float


class Model(C.Structure):
    _fields_ = [
        ("num_vertices", I32), ("num_tetrahedrons", I32), ("num_edges", I32), ("num_triangles", I32),
        ("num_connectors", I32), ("num_envs", I32),
        ("vertex", P), ("predicted_vertex", P), ("velocity", P), ("dp", P), ("constraints_number", P),
        ("collision_dp", P), ("inverse_mass", P),
        ("tetrahedron", P), ("tetrahedron_rest_volume", P), ("active_tetrahedron", P), ("tetrahedron_dm_inv", P),
        ("tetrahedron_lambda", P), ("xpbd_rest_volume", P),
        ("edge", P), ("edge_rest_length", P), ("active_edge", P), ("edge_lambda", P),
        ("triangle", P), ("tri_to_env", P), ("hole", P), ("vertex_to_env", P), ("active_drag_constraint", P),
        ("laparoscope_base", P), ("laparoscope_tip", P), ("laparoscope_radius", P), ("laparoscope_in_collision", P),
        ("connector_triangle_id", P), ("connector_tri_bar", P), ("connector_vertex_id", P), ("connector_rest_dist", P),
        ("env_vertex_start", P), ("env_tet_start", P), ("env_edge_start", P), ("env_tri_start", P),
    ]


class Params(C.Structure):
    _fields_ = [
        ("substeps", I32), ("iterations", I32), ("flags", C.c_uint32), ("dt", F32), ("gravity", F32 * 3),
        ("velocity_dampening", F32), ("ground_level", F32),
        ("ks_distance", F32), ("ks_volume", F32), ("ks_contact", F32), ("ks_drag", F32),
        ("volume_compliance", F32), ("deviatoric_compliance", F32),
        ("distance_compliance", F32), ("volume_compliance_xpbd", F32),
        ("connector_mass_weight_ratio", F32), ("connector_ks", F32), ("connector_rest_length_mul", F32),
    ]


class Bvh(C.Structure):
    _fields_ = [
        ("num_envs", I32), ("num_topologies", I32),
        ("env_topology", P), ("env_node_offset", P), ("env_face_offset", P),
        ("topo_node_offset", P), ("topo_tri_offset", P), ("topo_max_level", P),
        ("left_node", P), ("first_tri_id", P), ("tri_count", P), ("level", P), ("tri_id", P),
        ("aabb_min", P), ("aabb_max", P),
        ("total_env_nodes", I32), ("total_topology_nodes", I32), ("max_level", I32),
        ("level_node", P), ("level_start", P), ("topo_level_offset", P), ("node_box", P), ("tri_pos", P),
        ("refit_source", P),
    ]


class Render(C.Structure):
    _fields_ = [
        ("num_envs", I32), ("resolution", I32), ("num_vis_points", I32), ("num_vis_faces", I32),
        ("vis_point", P), ("vis_face", P), ("vis_point_color", P), ("normal_sum", P), ("vertex_normal", P),
        ("point_face_start", P), ("point_face", P),
        ("num_cameras", I32), ("camera_pos", P), ("camera_rot", P), ("camera_tan", F32), ("camera_aspect", F32),
        ("num_lights", I32), ("light_dir", P), ("light_intensity", P),
        ("color", P), ("depth", P), ("rays", P), ("ray_depth", P), ("error_flag", P), ("env_point_start", P),
        ("render_mode", I32), ("texture", P), ("env_objects", P), ("object_texture", P), ("tex_coords", P),
        ("tex_indices", P),
    ]


class RenderConfig(C.Structure):
    """ffsrl_render_config of include/ffsrl.h."""
    _fields_ = [("num_points", I32), ("num_faces", I32), ("points", P), ("faces", P), ("colors", P),
                ("num_map", I32), ("point_to_vertex", P), ("env_point_start", P), ("env_face_start", P),
                ("env_topology", P), ("resolution", I32), ("camera_tan", F32), ("camera_aspect", F32),
                ("num_lights", I32), ("light_dir", P), ("light_intensity", P), ("render_mode", I32)]


class ServerConfig(C.Structure):
    """ffsrl_server_config of include/ffsrl.h."""
    _fields_ = [("num_slots", I32), ("slot_mesh", P), ("num_actors", I32), ("actor_mesh", P), ("lanes", I32),
                ("plan", P), ("model", C.POINTER(Model)), ("initial_vertex", P), ("initial_base", P),
                ("initial_tip", P), ("xform", P), ("initial_xform", P), ("height", P), ("grasp_cand_start", P),
                ("grasp_cand", P), ("grasp_radius", F32), ("vis_point", P), ("point_to_vertex", P),
                ("env_map_start", P), ("inst_local_point", P), ("inst_point_slot", P), ("inst_num_points", I32),
                ("env_inst_first_point", P), ("bvh", C.POINTER(Bvh)), ("vis_face", P), ("render", C.POINTER(Render))]


# ffsrl_batch_options.arithmetic / .accumulation
ARITH_REFERENCE = 0
ARITH_FAST = 1
ACC_FIXED = 0
ACC_KAHAN = 1
ACC_ATOMIC = 2


class BatchOptions(C.Structure):
    _fields_ = [("block_threads", I32), ("arithmetic", I32), ("accumulation", I32), ("precision", I32),
                ("reserved", I32 * 4)]


_lib = None


def lib() -> C.CDLL:
    """The loaded library; raises FFSRLError when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        raise FFSRLError(ERR_UNSUPPORTED, f"{_LIB_PATH.name} is not built; run __graft_entry__.build() "
                                          "or python ff-srl_gb300/ffsrl/_build.py")
    L = C.CDLL(str(_LIB_PATH))
    pm, pp, pb, pr = C.POINTER(Model), C.POINTER(Params), C.POINTER(Bvh), C.POINTER(Render)
    sig = {
        "ffsrl_abi_version": ([], I32),
        "ffsrl_last_error": ([], C.c_char_p),
        "ffsrl_device_info": ([C.POINTER(I32)] * 4, I32),
        "ffsrl_step_model": ([pm, pp, P], I32),
        "ffsrl_step_model_noalloc": ([pm, pp, P], I32),
        "ffsrl_remap": ([P, P, P, I32, P], I32),
        "ffsrl_remap_envs": ([P, P, P, P, P, I32, I32, P], I32),
        "ffsrl_update_clamps_drag": ([P, P, P, P, F32, P, P, I32, P], I32),
        "ffsrl_force_clamps_drag": ([P, I32, P, I32, F32, I32, P], I32),
        "ffsrl_grasp_nearest": ([P, P, P, P, P, F32, P, I32, P], I32),
        "ffsrl_move_tool": ([P, P, P, I32, P], I32),
        "ffsrl_move_tool_envs": ([P, P, P, P, I32, I32, P], I32),
        "ffsrl_reset_envs": ([P, P, P, P, P, P, P, P, P, P, P, P, P, I32, I32, P], I32),
        "ffsrl_instrument_update": ([P, P, P, P, I32, P], I32),
        "ffsrl_instrument_apply_actions": ([P, P, P, P, P, P, P, I32, P], I32),
        "ffsrl_instrument_cartesian": ([P, P, P, P, P, P, P, I32, P], I32),
        "ffsrl_instrument_cartesian_envs": ([P, P, P, P, P, P, P, P, I32, I32, P], I32),
        "ffsrl_instrument_set_rotation_center": ([P, P, P, P, P, P, I32, P], I32),
        "ffsrl_instrument_visual_update": ([P, P, P, I32, P, P, P, I32, I32, P], I32),
        "ffsrl_grasp_nearest_envs": ([P, P, P, P, P, F32, P, P, I32, I32, P], I32),
        "ffsrl_bvh_refit_fused_envs": ([pb, P, P, P, I32, P], I32),
        "ffsrl_render_fused_envs": ([pr, pb, P, I32, P], I32),
        "ffsrl_batch_step_envs_lane": ([P, I32, P, I32, I32, P], I32),
        "ffsrl_bvh_build_host": ([P, P, I32, I32, I32, P, P, P, P, P, P, P, C.POINTER(I32), C.POINTER(I32)], I32),
        "ffsrl_bvh_refit_levels": ([pb, P, P, P], I32),
        "ffsrl_bvh_refit_fused": ([pb, P, P, P], I32),
        "ffsrl_render_reference": ([pr, pb, P], I32),
        "ffsrl_render_fused": ([pr, pb, P], I32),
        "ffsrl_batch_create": ([pm, pm, pp, C.POINTER(BatchOptions), C.POINTER(P)], I32),
        "ffsrl_batch_destroy": ([P], I32),
        "ffsrl_batch_step": ([P, I32, P], I32),
        "ffsrl_batch_step_envs": ([P, P, I32, I32, P], I32),
        "ffsrl_batch_info": ([P, C.POINTER(C.c_int64), C.POINTER(I32), P], I32),
        "ffsrl_batch_env_status": ([P, P, I32], I32),
        "ffsrl_batch_state_f64": ([P, P], I32),
        "ffsrl_batch_class_info": ([P, I32, C.POINTER(I32), C.POINTER(I32), C.POINTER(I32), C.POINTER(I32)], I32),
        "ffsrl_batch_class_envs": ([P, I32, P], I32),
        "ffsrl_batch_set_class_block": ([P, I32, I32], I32),
        "ffsrl_batch_set_class_prefetch": ([P, I32, I32], I32),
        "ffsrl_create": ([pm, pp, I32, C.POINTER(P)], I32),
        "ffsrl_destroy": ([P], I32),
        "ffsrl_step": ([P, I32, P], I32),
        "ffsrl_get_device_model": ([P, pm, C.POINTER(P)], I32),
        "ffsrl_set_tool": ([P, P, P, P, I32, P], I32),
        "ffsrl_set_drag": ([P, P, I32, P], I32),
        "ffsrl_attach_render": ([P, C.POINTER(RenderConfig)], I32),
        "ffsrl_render_handle": ([P, P, P, I32, P, P, P], I32),
        "ffsrl_render_handle_check": ([P, P], I32),
        "ffsrl_server_create": ([C.POINTER(ServerConfig), C.POINTER(P)], I32),
        "ffsrl_server_destroy": ([P], I32),
        "ffsrl_server_submit": ([P, I32, P, I32, I32, C.c_int64], I32),
        "ffsrl_server_launch": ([P, I32, C.POINTER(I32)], I32),
        "ffsrl_server_poll": ([P, I32, P, P, P, C.POINTER(I32)], I32),
        "ffsrl_server_admit": ([P, I32, C.POINTER(I32)], I32),
        "ffsrl_server_evict": ([P, I32], I32),
        "ffsrl_server_stats": ([P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(I32), C.POINTER(I32)], I32),
        "ffsrl_graph_begin": ([P], I32),
        "ffsrl_graph_end": ([P, C.POINTER(P)], I32),
        "ffsrl_graph_launch": ([P, P], I32),
        "ffsrl_graph_destroy": ([P], I32),
        "ffsrl_edge_breaker": ([P, P, P, P, P, I32, F32, F32, P], I32),
        "ffsrl_check_edge_breaker": ([P, P, P, P, I32, P, I32, P, P, P, P, F32, P, P, P], I32),
        "ffsrl_tetrahedron_breaker": ([P, P, P, P, P, I32, F32, P], I32),
        "ffsrl_heat_propagation": ([P, P, P, P, I32, F32, F32, F32, P], I32),
        "ffsrl_heat_update": ([P, P, P, P, P, P, I32, I32, P], I32),
        "ffsrl_check_heat": ([P, P, P, P, P, F32, I32, P], I32),
        "ffsrl_heat_laparoscope": ([P, P, P, P, P, P, P, F32, F32, I32, P], I32),
        "ffsrl_cut_edges": ([P, P, P, P, P, I32, P, I32, P, P, P, P, P, P, P], I32),
        "ffsrl_update_active_values": ([P, P, P, I32, I32, P], I32),
    }
    for name, (args, ret) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ret
    _lib = L
    return L


def check(code: int) -> None:
    if code != OK:
        msg = lib().ffsrl_last_error()
        raise FFSRLError(code, msg.decode() if msg else "")


def ptr(t) -> int | None:
    """Address of a torch tensor's or numpy array's data (None for None)."""
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return t.data_ptr()
    return t.ctypes.data


def stream_handle(stream=None) -> int | None:
    """cudaStream_t of a torch stream (default: torch's current stream)."""
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream or None

"""ctypes mirror of the boundary types declared in include/ctbb_gb300.h.

The layout is the one of the reference's ``struct recon_metadata``
(include/recon_structs.h:26-113) and ``struct recon_params``
(include/parse_config.h:36-67): same field names, types and order, so the same
bytes can be handed to this library's C ABI or to the reference's functions.
"""
import ctypes as C

__all__ = [
    "ReconParams", "BlockInfo", "ReconInfo", "CtData", "CtGeom", "Flags",
    "ReconMetadata",
]


class ReconParams(C.Structure):
    _fields_ = [
        ("raw_data_dir", C.c_char * 4096),
        ("raw_data_file", C.c_char * 255),
        ("output_dir", C.c_char * 4096),
        ("output_file", C.c_char * 255),
        ("n_rows", C.c_int),
        ("coll_slicewidth", C.c_float),
        ("start_pos", C.c_float),
        ("end_pos", C.c_float),
        ("pitch_value", C.c_float),
        ("slice_thickness", C.c_float),
        ("acq_fov", C.c_float),
        ("recon_fov", C.c_float),
        ("recon_kernel", C.c_int),
        ("n_readings", C.c_int),
        ("x_origin", C.c_float),
        ("y_origin", C.c_float),
        ("z_ffs", C.c_int),
        ("phi_ffs", C.c_int),
        ("scanner", C.c_char * 4351),
        ("file_type", C.c_int),
        ("file_subtype", C.c_int),
        ("raw_data_offset", C.c_int),
        ("nx", C.c_uint),
        ("ny", C.c_uint),
        ("tube_start_angle", C.c_float),
        ("adaptive_filtration_s", C.c_float),
        ("n_slices", C.c_int),
        ("table_dir_str", C.c_char * 1024),
        ("table_dir", C.c_int),
    ]


class BlockInfo(C.Structure):
    _fields_ = [
        ("block_idx", C.c_int),
        ("block_slice_start", C.c_float),
        ("block_slice_end", C.c_float),
        ("idx_block_slice_start", C.c_int),
        ("idx_block_slice_end", C.c_int),
    ]


class ReconInfo(C.Structure):
    _fields_ = [
        ("n_ffs", C.c_size_t),
        ("data_begin_pos", C.c_float),
        ("data_end_pos", C.c_float),
        ("allowed_begin", C.c_float),
        ("allowed_end", C.c_float),
        ("n_slices_requested", C.c_size_t),
        ("n_slices_recon", C.c_size_t),
        ("n_slices_block", C.c_size_t),
        ("n_blocks", C.c_size_t),
        ("idx_slice_start", C.c_size_t),
        ("idx_slice_end", C.c_size_t),
        ("recon_start_pos", C.c_float),
        ("recon_end_pos", C.c_float),
        ("idx_pull_start", C.c_size_t),
        ("idx_pull_end", C.c_size_t),
        ("n_proj_pull", C.c_size_t),
        ("cb", BlockInfo),
    ]


class CtData(C.Structure):
    _fields_ = [
        ("raw", C.POINTER(C.c_float)),
        ("rebin", C.POINTER(C.c_float)),
        ("image", C.POINTER(C.c_float)),
        ("d_raw", C.c_void_p),
        ("d_rebin", C.c_void_p),
        ("d_image", C.c_void_p),
        ("d_final_image_stack", C.c_void_p),
        ("final_image_stack", C.POINTER(C.c_float)),
    ]


class CtGeom(C.Structure):
    _fields_ = [
        ("n_proj_turn", C.c_size_t),
        ("n_proj_ffs", C.c_size_t),
        ("n_channels", C.c_size_t),
        ("n_channels_oversampled", C.c_size_t),
        ("n_rows", C.c_size_t),
        ("n_rows_raw", C.c_size_t),
        ("r_f", C.c_float),
        ("z_rot", C.c_float),
        ("theta_cone", C.c_float),
        ("fan_angle_increment", C.c_float),
        ("src_to_det", C.c_float),
        ("anode_angle", C.c_float),
        ("central_channel", C.c_float),
        ("acq_fov", C.c_float),
        ("projection_offset", C.c_size_t),
        ("add_projections", C.c_size_t),
        ("add_projections_ffs", C.c_size_t),
        ("reverse_row_interleave", C.c_int),
        ("reverse_channel_interleave", C.c_int),
        ("table_direction", C.c_int),
    ]


class Flags(C.Structure):
    _fields_ = [
        ("testing", C.c_int),
        ("verbose", C.c_int),
        ("no_gpu", C.c_int),
        ("set_device", C.c_int),
        ("device_number", C.c_int),
        ("timing", C.c_int),
        ("benchmark", C.c_int),
    ]


class ReconMetadata(C.Structure):
    _fields_ = [
        ("home_dir", C.c_char * 4096),
        ("cwd", C.c_char * 4096),
        ("install_dir", C.c_char * 4096),
        ("flags", Flags),
        ("rp", ReconParams),
        ("ri", ReconInfo),
        ("cg", CtGeom),
        ("ctd", CtData),
        ("tube_angles", C.POINTER(C.c_float)),
        ("table_positions", C.POINTER(C.c_double)),
    ]


def layout_offsets():
    """Offsets checked against the reference build and the C header."""
    return [
        ReconMetadata.flags.offset, ReconMetadata.rp.offset, ReconMetadata.ri.offset,
        ReconMetadata.cg.offset, ReconMetadata.ctd.offset,
        ReconMetadata.tube_angles.offset, ReconMetadata.table_positions.offset,
        ReconParams.nx.offset, ReconParams.table_dir.offset, ReconInfo.cb.offset,
        CtGeom.table_direction.offset,
    ]


class RequestResult(C.Structure):
    """struct ctbb_request_result (a finished server request)."""
    _fields_ = [
        ("status", C.c_int), ("worker", C.c_int), ("device_bytes", C.c_size_t),
        ("queue_ms", C.c_double), ("run_ms", C.c_double), ("latency_ms", C.c_double),
        ("start_ms", C.c_double), ("end_ms", C.c_double),
        ("error", C.c_char * 256),
    ]

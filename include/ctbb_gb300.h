/*
 * ctbb_gb300.h -- C ABI of the GB300 helical weighted-FBP library.
 *
 * Two layers are declared here.
 *
 *  1. The boundary types.  struct recon_params, struct recon_info, struct ct_data,
 *     struct ct_geom, struct flags and struct recon_metadata have the same field
 *     names, types and order as the CTBangBang types they stand in for
 *     (include/parse_config.h:36-67 and include/recon_structs.h:26-113 of the
 *     reference), so a driver written against the reference's headers passes the
 *     same bytes to this library.
 *
 *  2. Entry points.  Every extern "C" function returns a ctbb_status (0 = success)
 *     and never calls exit().  Under C++ the header also declares the four
 *     reference module functions with their original C++ linkage
 *     (adaptive_filter_kk, rebin_filter, backproject, finalize_image_stack), so a
 *     driver that follows the reference main.cu call order links unchanged.
 *
 * Data layouts (all float32, C order, fastest index last):
 *   raw     [n_proj_pull][n_rows_raw][n_channels]              host, ctd.raw
 *   rebin   [n_views][n_rows][n_channels_oversampled]           device, ctd.d_rebin
 *           n_views = n_proj_pull/n_ffs - 2*add_projections
 *   image   [n_slices_recon][ny][nx]                            host, ctd.image
 *   final   [n_slices_final][ny][nx]                            host, ctd.final_image_stack
 *
 * Threading: calls on one recon_metadata are not reentrant (the reference's are
 * not either).  Device work runs on the stream set by ctbb_set_stream (default:
 * the legacy default stream) and every drop-in call returns after that stream is
 * synchronised, as the reference's blocking cudaMemcpy calls did.
 */
#ifndef CTBB_GB300_H
#define CTBB_GB300_H

#include <stddef.h>
#include <stdint.h>

/* ------------------------------------------------------------------------- */
/* Boundary types (layout of the reference's parse_config.h / recon_structs.h) */
/* ------------------------------------------------------------------------- */

/* A driver that already included the reference's parse_config.h /
   recon_structs.h (include guards parse_config_h / recon_structs_h) keeps its
   own identical definitions. */
#if !defined(parse_config_h)
/* .prm keys, parse_config.h:36-67 of the reference. */
struct recon_params {
    char raw_data_dir[4096];
    char raw_data_file[255];
    char output_dir[4096];
    char output_file[255];
    int n_rows;                 /* Nrows: detector rows after z-FFS            */
    float coll_slicewidth;      /* CollSlicewidth [mm at isocentre]            */
    float start_pos;            /* StartPos [mm]                               */
    float end_pos;              /* EndPos [mm]                                 */
    float pitch_value;          /* PitchValue / TableFeed: feed per turn [mm]  */
    float slice_thickness;      /* SliceThickness [mm]                         */
    float acq_fov;              /* AcqFOV [mm]                                 */
    float recon_fov;            /* ReconFOV [mm]                               */
    int recon_kernel;           /* ReconKernel: -100 ramp, -1,1,2,3, else b<k> */
    int n_readings;             /* Readings: frames in the raw file            */
    float x_origin;             /* Xorigin [mm]                                */
    float y_origin;             /* Yorigin [mm]                                */
    int z_ffs;                  /* Zffs                                        */
    int phi_ffs;                /* Phiffs                                      */
    char scanner[4351];         /* Scanner: .scanner path or 0/1/2             */
    int file_type;              /* FileType (0 = float32 binary frames)        */
    int file_subtype;           /* FileSubType                                 */
    int raw_data_offset;        /* RawOffset [bytes]                           */
    unsigned int nx;            /* Nx                                          */
    unsigned int ny;            /* Ny                                          */
    float tube_start_angle;     /* TubeStartAngle [deg]                        */
    float adaptive_filtration_s;/* AdaptiveFiltration strength                 */
    int n_slices;               /* NSlices (overrides EndPos when non-zero)    */
    char table_dir_str[1024];   /* TableDir: "in" / "out"                      */
    int table_dir;              /* TableDirInt: -1 in, 1 out                   */
};
#endif /* parse_config_h */

#if !defined(recon_structs_h)
struct block_info {
    int block_idx;
    float block_slice_start;
    float block_slice_end;
    int idx_block_slice_start;
    int idx_block_slice_end;
};

struct recon_info {
    size_t n_ffs;
    float data_begin_pos;
    float data_end_pos;
    float allowed_begin;
    float allowed_end;
    size_t n_slices_requested;
    size_t n_slices_recon;
    size_t n_slices_block;
    size_t n_blocks;
    size_t idx_slice_start;
    size_t idx_slice_end;
    float recon_start_pos;
    float recon_end_pos;
    size_t idx_pull_start;
    size_t idx_pull_end;
    size_t n_proj_pull;
    struct block_info cb;
};

struct ct_data {
    float *raw;
    float *rebin;
    float *image;
    float *d_raw;
    float *d_rebin;
    float *d_image;
    float *d_final_image_stack;
    float *final_image_stack;
};

struct ct_geom {
    size_t n_proj_turn;
    size_t n_proj_ffs;
    size_t n_channels;
    size_t n_channels_oversampled;
    size_t n_rows;
    size_t n_rows_raw;
    float r_f;
    float z_rot;
    float theta_cone;
    float fan_angle_increment;
    float src_to_det;
    float anode_angle;
    float central_channel;
    float acq_fov;
    size_t projection_offset;
    size_t add_projections;
    size_t add_projections_ffs;
    int reverse_row_interleave;
    int reverse_channel_interleave;
    int table_direction;        /* -1 table positions decreasing, 1 increasing */
};

struct flags {
    int testing;
    int verbose;
    int no_gpu;
    int set_device;
    int device_number;
    int timing;
    int benchmark;
};

struct recon_metadata {
    char home_dir[4096];
    char cwd[4096];
    char install_dir[4096];
    struct flags flags;
    struct recon_params rp;
    struct recon_info ri;
    struct ct_geom cg;
    struct ct_data ctd;
    float *tube_angles;
    double *table_positions;
};

#endif /* recon_structs_h */

/* ------------------------------------------------------------------------- */
/* Status codes                                                              */
/* ------------------------------------------------------------------------- */

typedef enum ctbb_status {
    CTBB_OK = 0,
    CTBB_ERR_ARGUMENT = 1,      /* null pointer, zero size, unsupported value    */
    CTBB_ERR_CONFIG = 2,        /* .prm / .scanner key missing or inconsistent   */
    CTBB_ERR_RANGE = 3,         /* recon range outside the allowed data range    */
    CTBB_ERR_IO = 4,            /* file not found / short read / write failed    */
    CTBB_ERR_CUDA = 5,          /* a CUDA runtime call failed (see last error)   */
    CTBB_ERR_NO_DEVICE = 6,     /* no CUDA device: the library has no CPU path   */
    CTBB_ERR_ALLOC = 7,         /* host or device allocation failed              */
    CTBB_ERR_STATE = 8          /* call out of order (e.g. backproject w/o rebin) */
} ctbb_status;

#ifdef __cplusplus
extern "C" {
#endif

/* Human-readable text of the last error on this thread ("" if none). */
const char *ctbb_last_error(void);

/* Library version string. */
const char *ctbb_version(void);

/* sizeof(struct recon_metadata) followed by the offsets of its members flags,
   rp, ri, cg, ctd, tube_angles, table_positions and of recon_params.nx,
   recon_params.table_dir, recon_info.cb, ct_geom.table_direction, as compiled
   into the library (a binding checks its own struct mirror against these).
   Writes min(n, 12) values; returns 12. */
int ctbb_struct_layout(size_t *out, int n);

/* Stream on which all device work of the following calls is issued
   (a cudaStream_t passed as void*; NULL = legacy default stream).  The
   streamed whole-scan calls (ctbb_reconstruct_scan_host / _file) also use a
   copy stream and a preparation stream of the library's own, ordered after
   the work already on this stream and joined before they return. */
int ctbb_set_stream(void *stream);

/* ------------------------------------------------------------------------- */
/* Planner (host).  Bit-exact restatements of the reference's integer tables. */
/* ------------------------------------------------------------------------- */

/* Parse a .prm file into *rp and apply the TableDir defaults and the
   required-key checks.  Replaces configure_recon_params, src/setup.cu:108-176
   (and parse_config, src/parse_config.cu:40-217).  Returns CTBB_ERR_CONFIG
   instead of exit(1) when a required key is missing. */
int ctbb_configure_recon_params(const char *prm_path, struct recon_params *rp);

/* Fill mr->cg from mr->rp.scanner (a .scanner file path, a file name under
   <install_dir>/resources/scanners, or the built-in scanners "0", "1", "2").
   Replaces configure_ct_geom, src/setup.cu:178-383. */
int ctbb_configure_ct_geom(struct recon_metadata *mr);

/* Per-frame tube angle / table position tables for FileType 0, the recon slice
   range, block count and first pull window; allocates mr->tube_angles,
   mr->table_positions, mr->ctd.raw, mr->ctd.rebin and mr->ctd.image (calloc).
   Replaces configure_reconstruction, src/setup.cu:385-603.  The raw file is
   not opened; CTBB_ERR_RANGE replaces the reference's exit(1). */
int ctbb_configure_reconstruction(struct recon_metadata *mr);

/* Next 32-slice block: pull window, block slice range, block_idx++ and
   re-allocation of ctd.raw / ctd.rebin.  Replaces update_block_info,
   src/setup.cu:605-679. */
int ctbb_update_block_info(struct recon_metadata *mr);

/* Read the block's pull window of FileType-0 frames (float32, little endian,
   RawOffset bytes of header) into ctd.raw; frames past the end of the file read
   as zeros.  Replaces extract_projections, src/setup.cu:681-767 (type 0 only). */
int ctbb_extract_projections(struct recon_metadata *mr);

/* Write the float32 final stack to <output_dir>/<output_file> and free every
   host array the planner and finalize allocated.  Replaces finish_and_cleanup,
   src/setup.cu:769-787. */
int ctbb_finish_and_cleanup(struct recon_metadata *mr);

/* The final stack h_stack [n_slices][ny][nx] (host) as a DICOM CT image
   series, one file per slice, <out_dir>/<OutputFile stem>_<k+1, 4 digits>.dcm
   ("slice" when OutputFile is empty).  No counterpart in the reference, which
   writes the raw float32 stack (finish_and_cleanup, src/setup.cu:769-787).
   mu_water > 0: the stack holds attenuation (1/mm) and is written as
   1000 (mu - mu_water) / mu_water; mu_water = 0: it already holds HU.  Pixels
   are int16 HU (rounded, clamped), rescale slope 1, intercept 0; explicit VR
   little endian; pixel (i, j) at the backprojector's voxel centre, slice k at
   StartPos + dir k SliceThickness; fresh 2.25 study / series UIDs per call.
   No patient identity is written (PatientName and PatientID empty). */
int ctbb_write_dicom_series(const struct recon_metadata *mr, const float *h_stack,
                            int n_slices, float mu_water, const char *out_dir);

/* Number of final slices: floor(|end-start|/slice_thickness)+1
   (src/finalize_image_stack_cpu.cu:67). */
int ctbb_n_slices_final(const struct recon_metadata *mr);

/* Load the 2*n_channels_oversampled float32 reconstruction-kernel taps named by
   rp.recon_kernel from <install_dir>/resources/filters/f_<N>_<name>.txt.  For
   ReconKernel -100 a missing f_<N>_ramp.txt is generated from the ramp formula
   (ctbb_ramp_filter_taps).  Replaces load_filter, src/rebin_filter.cu:922-959. */
int ctbb_load_filter(const struct recon_metadata *mr, float *taps_out);

/* Ramp/apodised kernel taps f[j], j in [0, 2*n_os): f = (c^2/(2 ds)) *
   (a r(c pi k) + (1-a)/2 r(c pi k + pi) + (1-a)/2 r(c pi k - pi)), k = j - n_os,
   r(t) = sin t/t + (cos t - 1)/t^2, r(0) = 1/2, ds = r_f sin(fan_angle_inc/2)
   (resources/ramp.m of the reference). */
int ctbb_ramp_filter_taps(int n_os, float ds, float c, float a, float *taps_out);

/* ------------------------------------------------------------------------- */
/* Hot path: drop-in module functions (host buffers, reference semantics).    */
/* ------------------------------------------------------------------------- */

/* Kachelriess-Kalender adaptive raw-data filter on ctd.raw, in place.
   Replaces adaptive_filter_kk, src/preprocessing.cu:31-156 / include/preprocessing.h:26. */
int ctbb_adaptive_filter_kk(struct recon_metadata *mr);

/* FFS + fan-to-parallel rebinning and ramp filtering of ctd.raw.  The result is
   left on the device in ctd.d_rebin (cudaMalloc'd here, freed by
   ctbb_backproject), as the reference does.  If mr->flags.testing is set the
   result is also copied to the host array ctd.rebin.
   Replaces rebin_filter, src/rebin_filter.cu:38-56 / include/rebin_filter.h:27. */
int ctbb_rebin_filter(struct recon_metadata *mr);

/* Weighted-FBP backprojection of ctd.d_rebin into the 32-slice block
   ctd.image[(cb.block_idx-1)*nx*ny*32 ...], CPU-path conventions
   (src/backproject_cpu.cu:49-154).  Frees ctd.d_rebin.
   Replaces backproject, src/backproject.cu:31-108 / include/backproject.h:26. */
int ctbb_backproject(struct recon_metadata *mr);

/* Block reorder + triangle slice thickening of ctd.image into a newly
   calloc'd ctd.final_image_stack (attenuation units, as the reference).
   Replaces finalize_image_stack, src/finalize_image_stack.cu:26-120 /
   include/finalize_image_stack.h:26 (CPU twin src/finalize_image_stack_cpu.cu:24-117). */
int ctbb_finalize_image_stack(struct recon_metadata *mr);

/* As ctbb_finalize_image_stack, then HU = 1000 (mu - mu_water) / mu_water.
   No counterpart in the reference (it has no HU conversion). */
int ctbb_finalize_image_stack_hu(struct recon_metadata *mr, float mu_water);

/* ------------------------------------------------------------------------- */
/* Hot path: device-resident stages (device pointers, asynchronous on the     */
/* library stream).  These are what the drop-in functions call.              */
/* ------------------------------------------------------------------------- */

/* Adaptive filter of one pull window: d_raw_in -> d_raw_out (distinct buffers,
   [n_proj_pull][n_rows_raw][n_channels]).  Uses mr->cg, mr->ri, mr->rp. */
int ctbb_adaptive_filter_device(const struct recon_metadata *mr,
                                const float *d_raw_in, float *d_raw_out);

/* Adaptive filter of one pull window that allocates nothing.  No counterpart
   in the reference.  For callers that cannot allocate device memory while a
   scan is processed (a service that reserves all device memory at start-up
   and keeps cudaMalloc -- which can synchronise the device -- out of its
   per-scan path, or a process whose device memory belongs to another
   allocator): the per-frame statistics live in a fixed static device array of
   the library (6 floats per frame for at most 65536 frames, 1.5 MiB, held by
   every GPU that loads the library until the process exits) instead of the
   library's allocated workspace.  The caller passes d_raw_in and d_raw_out.
   Windows longer than 65536 frames are rejected with CTBB_ERR_ARGUMENT.  The
   first call on a device looks up the array's device address
   (cudaGetSymbolAddress), so make that first call before any stream capture.
   All calls share the array: calls that overlap on the GPU race.  Output is
   identical to ctbb_adaptive_filter_device. */
int ctbb_adaptive_filter_device_noalloc(const struct recon_metadata *mr,
                                        const float *d_raw_in, float *d_raw_out);

/* Rebin (no filter) of one pull window into d_rebin [n_views][n_rows][n_os]. */
int ctbb_rebin_device(const struct recon_metadata *mr, const float *d_raw,
                      float *d_rebin);

/* Ramp filter of n_lines rows of length n_os in place, taps of length 2*n_os. */
int ctbb_ramp_filter_device(float *d_lines, size_t n_lines, int n_os,
                            const float *h_taps);

/* Ramp filter of n_lines rows of length n_os (a multiple of 64, at most
   1536) as a Toeplitz contraction on the tensor cores: each product in FP16
   hi + lo halves (x_hi T_hi + x_hi T_lo + x_lo T_hi, x and T scaled by exact
   powers of two into FP16's range), accumulated in FP32.
   The result is stored as FP16 with a power-of-two scale per row, d_scale
   [n_lines]: y = stored value * d_scale.  rows_per_view = 0: d_out
   [n_lines][n_os] FP16 (2 bytes per sample), one scale per row.
   rows_per_view = R > 0 (R divides 128; lines are views of R detector rows):
   every row of a view has the view's scale, and d_out [n_lines][n_os][4] FP16
   holds each sample's bilinear footprint (y[r][c], y[r][c+1], y[r+1][c],
   y[r+1][c+1]) / scale, zero where r + 1 or c + 1 leaves the view (8 bytes
   per sample: one load per interpolation in the backprojector).  d_lines
   (float32, device) is not changed.  The same convolution as the reference's
   filter (include/rebin_filter.cuh:369-409) and filter_cpu
   (src/rebin_filter_cpu.cu:647-709); the reduced-storage path's filter. */
int ctbb_ramp_filter_fp16_device(const float *d_lines, size_t n_lines, int n_os, const float *h_taps,
                                 int rows_per_view, void *d_out, float *d_scale);

/* Backprojection of one block of filtered rebinned views into
   d_block [n_slices_block][ny][nx] (overwritten). */
int ctbb_backproject_device(const struct recon_metadata *mr,
                            const float *d_rebin, float *d_block);

/* ctbb_backproject_device from the reduced-storage rows: d_quads, the FP16
   footprint words of one block's views as ctbb_ramp_filter_fp16_device
   writes them with rows_per_view = n_rows ([n_views][n_rows][n_os][4]), and
   d_scale [n_views * n_rows] their scales (one per view); FP32 accumulation. */
int ctbb_backproject_fp16_device(const struct recon_metadata *mr, const void *d_quads, const float *d_scale,
                                 float *d_block);

/* Reorder + thicken d_image [n_slices_recon][ny][nx] into
   d_final [n_slices_final][ny][nx]; mu_water > 0 also converts to HU. */
int ctbb_finalize_device(const struct recon_metadata *mr, const float *d_image,
                         float *d_final, float mu_water);

/* Whole scan, device resident: every 32-slice block of the plan in *mr
   (re-planned with the reference's update_block_info per block) from the full
   raw scan d_scan [n_readings][n_rows_raw][n_channels] into
   d_final [n_slices_final][ny][nx].  mr->ri.cb.block_idx is reset to 0 first and
   advanced as in the reference block loop.  Work buffers are cached inside the
   library between calls. */
int ctbb_reconstruct_device(struct recon_metadata *mr, const float *d_scan,
                            float *d_final, float mu_water);

/* Whole scan from one resident rebinned scan (no counterpart in the
   reference, whose block loop pulls, filters and rebins each block's window
   separately although consecutive windows share most of their frames): the
   union of all blocks' pull windows is adaptive-filtered, rebinned and
   ramp-filtered once, and each block is backprojected from its offset into
   it.  Same plan, block order and output as ctbb_reconstruct_device.  The
   reference's adaptive filter stops its 18- and 180-degree statistics at
   each block's window ends, so the views a block reads from frames near those
   ends are re-made from the block's own window; the remaining difference to
   the block loop is the rounding of the rebin's view coordinate, which the
   union takes in split (integer + fraction) form (0.15 HU max over a
   40-turn scan of 13 blocks, 1472 x 128 rebinned rows).  Device memory: the union window's filtered raw
   data and rebinned rows, one block window and its re-made views. */
int ctbb_reconstruct_scan_device(struct recon_metadata *mr, const float *d_scan,
                                 float *d_final, float mu_water);

/* Many whole scans at once (no counterpart in the reference, which runs one
   scan per process): scan s of n_scans -- its own plan mrs[s], raw scan
   d_scans[s] and final stack d_finals[s], each as for
   ctbb_reconstruct_scan_device; the scans may differ in every geometry and
   size -- is filtered, rebinned and ramp-filtered into rows of its own, and
   then the 32-slice blocks of all scans are backprojected together, in one
   launch per launch shape, whose CTAs run over the tiles of every block in
   turn (short scans' small blocks fill the GPU beside one another).  The
   launch shape of each geometry class (image size, slices per block, row
   length, detector rows, half turns, row storage) is chosen by the
   autotuner: every candidate timed once on the first block of the class, the
   choice kept for the process (ctbb_autotune_report).  Row storage as set by
   ctbb_set_storage.  Each stack equals its scan's ctbb_reconstruct_scan_device
   result up to the launch shape's rounding (per-slice sums in another order).
   Device memory: every scan's rows, tables and image at once, plus one
   scan's window buffers (kept between calls; ctbb_release_workspace frees
   them).  mrs[s]->ri is left at the scan's last block. */
int ctbb_reconstruct_batch_device(int n_scans, struct recon_metadata *const *mrs, const float *const *d_scans,
                                  float *const *d_finals, float mu_water);

/* The same in steps, so that each raw scan can be freed once it is prepared:
   ctbb_batch_begin starts an empty batch; ctbb_batch_add_device prepares one
   scan (as ctbb_reconstruct_scan_device prepares it, into a slot of its own)
   and returns when d_scan is no longer read; ctbb_batch_run backprojects the
   blocks of every added scan and writes each final stack.  mr and d_final
   must stay valid until ctbb_batch_run returns. */
int ctbb_batch_begin(void);
int ctbb_batch_add_device(struct recon_metadata *mr, const float *d_scan, float *d_final, float mu_water);
int ctbb_batch_run(void);

/* on != 0: ctbb_reconstruct_scan_device on the library-wide context also
   takes the autotuner's launch shape for each block's geometry class (off by
   default: the measured default shape). */
int ctbb_set_autotune(int on);

/* The autotuner's choices so far, one text line per geometry class with the
   time of every candidate shape: writes min(n - 1, length) bytes and a NUL to
   buf, returns the full length. */
int ctbb_autotune_report(char *buf, size_t n);

/* ctbb_reconstruct_scan_device from host buffers, streamed (no counterpart in
   the reference): the union window is copied host->device in chunks on a
   second stream while each arriving chunk advances the adaptive filter as far
   as its statistics windows allow, views whose frames are final are rebinned
   and ramp-filtered, and each block is backprojected as soon as its views are
   ready.  Same result as ctbb_reconstruct_scan_device.  Pin h_scan
   (cudaHostRegister / cudaMallocHost) for the copies to overlap. */
int ctbb_reconstruct_scan_host(struct recon_metadata *mr, const float *h_scan,
                               float *h_final, float mu_water);

/* ctbb_reconstruct_scan_host reading the raw file of the plan itself (no
   counterpart in the reference, whose extract_projections reads each
   block's window again, src/setup.cu:681-767): a reader thread reads the
   union window of <RawDataDir>/<RawDataFile> (FileType 0: float32 frames at
   RawOffset + i * frame bytes; frames before the start or past the end of
   the file are zeros) in chunks into two pinned staging buffers (kept by the
   library, freed by ctbb_release_workspace) and enqueues each chunk's copy,
   while the compute stream works on the chunks that have arrived.  Other
   FileTypes return CTBB_ERR_CONFIG.  Same result as
   ctbb_reconstruct_scan_device on the file's frames. */
int ctbb_reconstruct_scan_file(struct recon_metadata *mr, float *h_final, float mu_water);

/* As ctbb_reconstruct_device from host buffers: each block's pull window is
   copied from h_scan [n_readings][n_rows_raw][n_channels] on a second stream
   (double-buffered, overlapping the previous block's compute when h_scan is
   pinned) and the final stack is copied to h_final [n_slices_final][ny][nx]. */
int ctbb_reconstruct_host(struct recon_metadata *mr, const float *h_scan, float *h_final,
                          float mu_water);

/* Row storage of the whole-scan paths (ctbb_reconstruct_scan_*), library-wide
   context: CTBB_STORAGE_FP32 (default) keeps the ramp-filtered rows in
   float32 (FFT convolution); CTBB_STORAGE_FP16 filters them on the tensor
   cores (ctbb_ramp_filter_fp16_device) into FP16 footprint words with one
   power-of-two scale per view, which the backprojector reads (one 8-byte
   load per interpolation), all voxel accumulation staying FP32.  FP16 needs
   rows of a multiple of 64 samples up to 1536 and detector rows dividing 128
   (else the reconstruction returns CTBB_ERR_ARGUMENT).  No counterpart in the
   reference, which keeps float32 rows. */
#define CTBB_STORAGE_FP32 0
#define CTBB_STORAGE_FP16 1
int ctbb_set_storage(int mode);

/* Per-stage device timing with CUDA events on the library stream.
   Stages: 0 adaptive filter, 1 rebin, 2 ramp filter, 3 backprojection,
   4 finalize.  ctbb_profile_read synchronises on the recorded events, adds
   their durations to per-stage totals, writes min(n, 5) totals (ms) and launch
   counts, optionally resets them, and returns 5. */
int ctbb_profile_enable(int on);
int ctbb_profile_read(double *ms, uint64_t *launches, int n, int reset);

/* Bytes of device workspace ctbb_reconstruct_device keeps for this plan. */
size_t ctbb_workspace_bytes(const struct recon_metadata *mr);

/* Release every cached device buffer, table, copy stream and event of the
   library (on the device they belong to) and unbind it from that device.
   The library's work buffers live on the device that was current at the
   first compute call; a call while another device is current returns
   CTBB_ERR_STATE until this function has been called. */
int ctbb_release_workspace(void);

/* Number of kernels this library launched since load (all entry points). */
uint64_t ctbb_kernel_launch_count(void);

/* ---- contexts: concurrent scans ----------------------------------------
   The reference keeps its state in per-translation-unit globals and runs one
   scan at a time.  Every entry point above uses one library-wide context
   (work buffers, tables, streams), serialised by a mutex.  A ctbb_context
   holds its own work buffers, tables and streams, so scans on different
   contexts run concurrently (from different host threads), their copies and
   kernels overlapping on the GPU; calls on one context are serialised.  The
   result of a scan does not depend on the context it ran on or on what runs
   beside it.  A context is bound to the device current at its creation and
   issues its work on a non-blocking stream of its own (or the caller's, after
   ctbb_context_set_stream).  No counterpart in the reference. */
typedef struct ctbb_context_s *ctbb_context;

int ctbb_context_create(ctbb_context *out);
/* Frees the context's device memory, streams and events; null is a no-op. */
int ctbb_context_destroy(ctbb_context ctx);
/* Issue the context's work on the caller's stream from now on. */
int ctbb_context_set_stream(ctbb_context ctx, void *stream);
/* ctbb_set_storage for the context's whole-scan calls. */
int ctbb_context_set_storage(ctbb_context ctx, int mode);
/* Frees the context's work buffers (kept and reused between calls otherwise). */
int ctbb_context_release_workspace(ctbb_context ctx);
/* Device bytes the context's work buffers hold now. */
size_t ctbb_context_device_bytes(ctbb_context ctx);
/* ctbb_reconstruct_scan_device / _scan_host / _scan_file / ctbb_reconstruct_device /
   ctbb_reconstruct_host on the context's buffers and stream. */
int ctbb_context_reconstruct_scan_device(ctbb_context ctx, struct recon_metadata *mr,
                                         const float *d_scan, float *d_final, float mu_water);
int ctbb_context_reconstruct_scan_host(ctbb_context ctx, struct recon_metadata *mr,
                                       const float *h_scan, float *h_final, float mu_water);
int ctbb_context_reconstruct_scan_file(ctbb_context ctx, struct recon_metadata *mr,
                                       float *h_final, float mu_water);
int ctbb_context_reconstruct_device(ctbb_context ctx, struct recon_metadata *mr,
                                    const float *d_scan, float *d_final, float mu_water);
int ctbb_context_reconstruct_host(ctbb_context ctx, struct recon_metadata *mr,
                                  const float *h_scan, float *h_final, float mu_water);

/* Device bytes the whole-scan entry points hold for this plan (the union
   window raw and filtered, its rebinned rows, the adaptive filter's
   statistics, the image and final stacks, 8 MiB of tables and slack); 0 if
   the plan is not usable.  Host only. */
size_t ctbb_scan_workspace_bytes(const struct recon_metadata *mr);

/* ---- request server: continuous batching of whole scans -----------------
   n_workers threads, each with its own context, take queued requests; a free
   worker starts the oldest request whose device memory
   (ctbb_scan_workspace_bytes) fits device_budget_bytes next to what the other
   workers hold (a request passed by younger ones for longer than the age
   bound of ctbb_server_configure is started before any other), so requests that arrive while others run are admitted as
   slots and memory free up and overlap them on the GPU.  Workers keep their
   buffers between requests; when a request does not fit, a worker drops its
   own buffers and asks idle workers to drop theirs.  Each request runs
   ctbb_context_reconstruct_scan_host: same result as ctbb_reconstruct_scan_host
   alone.  No counterpart in the reference. */
typedef struct ctbb_server_s *ctbb_server;

struct ctbb_request_result {
    int status;            /* ctbb_status of the reconstruction            */
    int worker;            /* worker that ran it                           */
    size_t device_bytes;   /* the request's device memory in the budget    */
    double queue_ms;       /* submission -> start                          */
    double run_ms;         /* start -> end                                 */
    double latency_ms;     /* submission -> end                            */
    double start_ms;       /* start, in ms since the server was created    */
    double end_ms;         /* end, same clock                              */
    char error[256];       /* ctbb_last_error() of a failed request        */
};

int ctbb_server_create(int n_workers, size_t device_budget_bytes, ctbb_server *out);
/* Row storage of the workers' reconstructions (CTBB_STORAGE_FP32 or
   CTBB_STORAGE_FP16, see ctbb_set_storage) and the age bound (ms): a queued
   request that does not fit the budget yet is passed by later requests that
   do, until it has waited that long (0: strict first in first out).  Call
   between requests. */
int ctbb_server_configure(ctbb_server srv, int storage, double age_bound_ms);
/* Requests started ahead of an older queued one so far. */
uint64_t ctbb_server_passed_count(ctbb_server srv);
/* Queue one scan: mr planned (configure_*; not shared with another request in
   flight), h_scan [n_readings][n_rows_raw][n_channels] (pinned host memory
   lets the copies overlap), h_final [n_slices_final][ny][nx].  A scan needing
   more than the budget is refused (CTBB_ERR_ALLOC). */
int ctbb_server_submit(ctbb_server srv, struct recon_metadata *mr, const float *h_scan,
                       float *h_final, float mu_water, uint64_t *ticket);
/* Block until the request is done; returns its status (and fills *out if
   not null).  Each ticket is waited for once. */
int ctbb_server_wait(ctbb_server srv, uint64_t ticket, struct ctbb_request_result *out);
/* Finish the queued requests, let threads blocked in ctbb_server_wait take
   their results, stop the workers, free their contexts.  No call on srv may
   start after this one. */
int ctbb_server_destroy(ctbb_server srv);

#ifdef __cplusplus
} /* extern "C" */

/* C++-linkage drop-ins with the reference's exact signatures. */
int adaptive_filter_kk(struct recon_metadata *mr);   /* include/preprocessing.h:26 */
int rebin_filter(struct recon_metadata *mr);         /* include/rebin_filter.h:27 */
int backproject(struct recon_metadata *mr);          /* include/backproject.h:26 */
int finalize_image_stack(struct recon_metadata *mr); /* include/finalize_image_stack.h:26 */
#endif

#endif /* CTBB_GB300_H */

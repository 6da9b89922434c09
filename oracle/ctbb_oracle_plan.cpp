// ctbb_oracle_plan.cpp -- TEST INFRASTRUCTURE: a CPU restatement of the
// reference's planner and configuration readers, so that a CPU run of the
// reference path (the benchmark's reference arm, the tests) can plan a scan
// without the reconstruction library.  Written after the reference sources:
//
//   oracle_configure_recon_params   parse_config (src/parse_config.cu:40-217)
//                                   + configure_recon_params (src/setup.cu:108-176)
//   oracle_configure_ct_geom        configure_ct_geom (src/setup.cu:178-383)
//   oracle_configure_reconstruction configure_reconstruction (src/setup.cu:385-603),
//                                   FileType 0 tables only; no host arrays for
//                                   the raw window / rebin / image are allocated
//   oracle_update_block_info        update_block_info (src/setup.cu:605-679),
//                                   without the host re-allocation
//   oracle_ramp_taps                resources/ramp.m
//
// Each keeps the reference's types, promotions and operation order, so the
// integer tables and float positions equal the reference build's
// (tests/test_cpu_oracle.py checks them against the golden plans the
// reference build wrote).  Failures return non-zero instead of exit().
#include <math.h>  // as the reference build: float overloads of fabs, floor, atan, fmod in the global namespace
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../include/ctbb_gb300.h"

namespace {

const float pi = 3.1415926535897f;  // src/setup.cu:33
const int kBlockSlices = 32;        // BLOCK_SLICES, src/setup.cu:34

// array_search, src/setup.cu:806-825
int array_search(float key, const double *array, int numel_array, int search_type)
{
    int idx = 0;
    switch (search_type) {
    case -1:
        while (idx < numel_array && key < array[idx]) idx++;
        break;
    case 0:
        while (idx < numel_array && key != array[idx]) idx++;
        break;
    case 1:
        while (idx < numel_array && key > array[idx]) idx++;
        break;
    }
    return idx;
}

// The pull window of a slice range (src/setup.cu:564-590 and :637-668).
void pull_window(const struct ct_geom &cg, int n_ffs, int idx_a, int idx_b, int *pull_start, int *pull_end,
                 int *n_pull)
{
    int pre_post_buffer = cg.n_proj_ffs / 2;
    int s, e;
    int lo = idx_a > idx_b ? idx_b : idx_a;
    int hi = idx_a > idx_b ? idx_a : idx_b;
    s = lo - pre_post_buffer - (int)cg.add_projections_ffs;
    s = (s - 1) + (n_ffs - (s - 1) % n_ffs);
    e = hi + pre_post_buffer + (int)cg.add_projections_ffs;
    e = (e - 1) + (n_ffs - (e - 1) % n_ffs);
    e += 256;
    int n = e - s;
    n = (n - 1) + (128 - (n - 1) % 128);
    *pull_start = s;
    *pull_end = s + n;
    *n_pull = n;
}

}  // namespace

extern "C" {

// parse_config + configure_recon_params: 0, or 2 when a required key is
// missing (the reference exits), 4 when the file cannot be read.
int oracle_configure_recon_params(const char *path, struct recon_params *p)
{
    memset(p, 0, sizeof(*p));
    FILE *f = fopen(path, "r");
    if (!f) return 4;
    char raw_line[1024], line[1024];
    while (fgets(raw_line, sizeof(raw_line), f)) {
        const char *pct = strchr(raw_line, '%');
        size_t n = pct ? (size_t)(pct - raw_line) : strlen(raw_line);
        memcpy(line, raw_line, n);
        line[n] = 0;
        if (line[0] == 0 || strcmp(line, "\n") == 0) continue;
        char *save = nullptr;
        char *key = strtok_r(line, " \t", &save);
        if (!key) continue;
        char *val = strtok_r(nullptr, " \t", &save);
        if (!val) continue;
#define S(k, field) else if (strcmp(key, k) == 0) sscanf(val, "%s", p->field)
#define I(k, field) else if (strcmp(key, k) == 0) sscanf(val, "%d", &p->field)
#define U(k, field) else if (strcmp(key, k) == 0) sscanf(val, "%u", &p->field)
#define F(k, field) else if (strcmp(key, k) == 0) sscanf(val, "%f", &p->field)
        if (0) {}
        S("RawDataDir:", raw_data_dir); S("RawDataFile:", raw_data_file);
        S("OutputDir:", output_dir); S("OutputFile:", output_file);
        I("Nrows:", n_rows); F("CollSlicewidth:", coll_slicewidth);
        F("StartPos:", start_pos); F("EndPos:", end_pos);
        F("TableFeed:", pitch_value); F("PitchValue:", pitch_value);
        F("SliceThickness:", slice_thickness); F("AcqFOV:", acq_fov); F("ReconFOV:", recon_fov);
        I("ReconKernel:", recon_kernel); I("Readings:", n_readings);
        F("Xorigin:", x_origin); F("Yorigin:", y_origin);
        I("Zffs:", z_ffs); I("Phiffs:", phi_ffs); S("Scanner:", scanner);
        I("FileType:", file_type); I("FileSubType:", file_subtype); I("RawOffset:", raw_data_offset);
        U("Nx:", nx); U("Ny:", ny); F("TubeStartAngle:", tube_start_angle);
        F("AdaptiveFiltration:", adaptive_filtration_s); I("NSlices:", n_slices);
        S("TableDir:", table_dir_str); I("TableDirInt:", table_dir);
#undef S
#undef I
#undef U
#undef F
    }
    fclose(f);
    if (strcmp(p->table_dir_str, "") != 0) {
        if (strcmp(p->table_dir_str, "out") == 0) p->table_dir = 1;
        else if (strcmp(p->table_dir_str, "in") == 0) p->table_dir = -1;
        else p->table_dir = 1;
    }
    if (p->n_rows == 0 || p->coll_slicewidth == 0 || p->slice_thickness == 0 || p->pitch_value == 0 ||
        p->acq_fov == 0 || p->recon_fov == 0 || p->n_readings == 0 || p->nx == 0 || p->ny == 0)
        return 2;
    if (p->file_type == 0 && p->table_dir == 0) p->table_dir = 1;
    return 0;
}

// configure_ct_geom: 0, or 2 when the scanner can be neither read nor parsed
// as a built-in number.
int oracle_configure_ct_geom(struct recon_metadata *mr)
{
    struct ct_geom cg;
    struct recon_params rp = mr->rp;
    memset(&cg, 0, sizeof(cg));
    cg.table_direction = rp.table_dir;
    int scanner = -1;
    FILE *f = fopen(mr->rp.scanner, "r");
    if (!f) {
        char path[4096 + 4400];
        snprintf(path, sizeof(path), "%s/resources/scanners/%s", mr->install_dir, mr->rp.scanner);
        f = fopen(path, "r");
        if (!f) {
            scanner = atoi(mr->rp.scanner);
            if ((scanner < 0 || scanner > 2) || (scanner == 0 && strlen(mr->rp.scanner) != 1)) return 2;
            if (scanner == 1) mr->rp.file_subtype = 1;
            if (scanner == 2) mr->rp.file_subtype = 2;
        }
    }
    if (scanner == -1) {
        fseek(f, 0, SEEK_END);
        size_t size = (size_t)ftell(f);
        rewind(f);
        char *buf = (char *)malloc(size + 1);
        buf[size] = 0;
        size_t got = fread(buf, 1, size, f);
        buf[got] = 0;
        fclose(f);
        char *save = nullptr;
        for (char *tok = strtok_r(buf, " \t\n%", &save); tok; tok = strtok_r(nullptr, " \t\n%", &save)) {
            char *v = nullptr;
            if (strcmp(tok, "RSrcToIso:") == 0) { if ((v = strtok_r(nullptr, " \t\n%", &save))) sscanf(v, "%f", &cg.r_f); }
            else if (strcmp(tok, "RSrcToDet:") == 0) { if ((v = strtok_r(nullptr, " \t\n%", &save))) sscanf(v, "%f", &cg.src_to_det); }
            else if (strcmp(tok, "AnodeAngle:") == 0) { if ((v = strtok_r(nullptr, " \t\n%", &save))) sscanf(v, "%f", &cg.anode_angle); }
            else if (strcmp(tok, "FanAngleInc:") == 0) { if ((v = strtok_r(nullptr, " \t\n%", &save))) sscanf(v, "%f", &cg.fan_angle_increment); }
            else if (strcmp(tok, "ThetaCone:") == 0) { if ((v = strtok_r(nullptr, " \t\n%", &save))) sscanf(v, "%f", &cg.theta_cone); }
            else if (strcmp(tok, "CentralChannel:") == 0) { if ((v = strtok_r(nullptr, " \t\n%", &save))) sscanf(v, "%f", &cg.central_channel); }
            else if (strcmp(tok, "NProjTurn:") == 0) { if ((v = strtok_r(nullptr, " \t\n%", &save))) sscanf(v, "%zu", &cg.n_proj_turn); }
            else if (strcmp(tok, "NChannels:") == 0) { if ((v = strtok_r(nullptr, " \t\n%", &save))) sscanf(v, "%zu", &cg.n_channels); }
            else if (strcmp(tok, "ReverseRowInterleave:") == 0) { if ((v = strtok_r(nullptr, " \t\n%", &save))) sscanf(v, "%i", &cg.reverse_row_interleave); }
            else if (strcmp(tok, "ReverseChanInterleave:") == 0) { if ((v = strtok_r(nullptr, " \t\n%", &save))) sscanf(v, "%i", &cg.reverse_channel_interleave); }
        }
        free(buf);
    } else if (scanner == 0) {  // src/setup.cu:300-321
        cg.r_f = 570.0f;
        cg.src_to_det = 1040.0f;
        cg.anode_angle = 7.0f * pi / 180.0f;
        cg.fan_angle_increment = 1.4083f / cg.src_to_det;
        cg.theta_cone = 2.0f * atan(7.5f * 1.3684f / cg.src_to_det);
        cg.central_channel = 335.25f;
        cg.n_proj_turn = 1160;
        cg.n_channels = 672;
    } else if (scanner == 1) {  // :323-346
        cg.r_f = 595.0f;
        cg.src_to_det = 1085.6f;
        cg.anode_angle = 7.0f * pi / 180.0f;
        cg.fan_angle_increment = 0.067864f * pi / 180.0f;
        cg.theta_cone = 2.0f * atan(7.5f * 1.2f / cg.r_f);
        cg.central_channel = 366.25f;
        cg.n_proj_turn = 1152;
        cg.n_channels = 736;
    } else {  // :348-372
        cg.r_f = 570.0f;
        cg.src_to_det = 1040.0f;
        cg.anode_angle = 7.0f * pi / 180.0f;
        cg.fan_angle_increment = 0.07758621f * pi / 180.0f;
        cg.theta_cone = 2.0f * atan(7.5f * 1.2f / cg.r_f);
        cg.central_channel = 334.25f;
        cg.n_proj_turn = 1160;
        cg.n_channels = 672;
    }
    // the derived quantities every case sets the same way (:285-292)
    cg.n_proj_ffs = cg.n_proj_turn * pow(2, rp.phi_ffs) * pow(2, rp.z_ffs);
    cg.n_channels_oversampled = 2 * cg.n_channels;
    cg.n_rows = (unsigned int)rp.n_rows;
    cg.n_rows_raw = (unsigned int)(rp.n_rows / pow(2, rp.z_ffs));
    cg.z_rot = rp.pitch_value;
    cg.add_projections = (cg.fan_angle_increment * cg.n_channels / 2) / (2.0f * pi / cg.n_proj_turn) + 10;
    cg.add_projections_ffs = cg.add_projections * pow(2, rp.z_ffs) * pow(2, rp.phi_ffs);
    cg.acq_fov = rp.acq_fov;
    if (rp.phi_ffs == 1) cg.central_channel = floor(cg.central_channel) + 0.375f;
    mr->cg = cg;
    return 0;
}

// configure_reconstruction for FileType 0: allocates (calloc) and fills
// mr->tube_angles / mr->table_positions and the recon_info ranges; 3 when
// the requested range lies outside the allowed data range.
int oracle_configure_reconstruction(struct recon_metadata *mr)
{
    struct ct_geom cg = mr->cg;
    struct recon_params rp = mr->rp;
    if (rp.file_type != 0 || rp.n_readings <= 100) return 2;
    mr->tube_angles = (float *)calloc(rp.n_readings, sizeof(float));
    mr->table_positions = (double *)calloc(rp.n_readings, sizeof(double));
    for (int i = 0; i < rp.n_readings; i++) {  // :399-410
        mr->tube_angles[i] = fmod(((360.0f / cg.n_proj_ffs) * i + rp.tube_start_angle), 360.0f);
        if (cg.table_direction == -1)
            mr->table_positions[i] = ((float)rp.n_readings / (float)cg.n_proj_ffs) * cg.z_rot -
                                     (float)i * cg.z_rot / (float)cg.n_proj_ffs;
        else
            mr->table_positions[i] = 0.0f + (float)i * cg.z_rot / (float)cg.n_proj_ffs;
    }
    int n_ffs = pow(2, rp.z_ffs) * pow(2, rp.phi_ffs);  // :484-530
    int n_slices_block = kBlockSlices;
    int recon_direction = fabs(rp.end_pos - rp.start_pos) / (rp.end_pos - rp.start_pos);
    if (recon_direction != 1 && recon_direction != -1) recon_direction = 1;
    if (rp.n_slices != 0) rp.end_pos = rp.start_pos + (rp.n_slices - 1) * rp.slice_thickness;
    float recon_start_pos = rp.start_pos - recon_direction * rp.slice_thickness;
    float recon_end_pos = rp.end_pos + recon_direction * rp.slice_thickness;
    int n_slices_requested = floor(fabs(recon_end_pos - recon_start_pos) / rp.coll_slicewidth) + 1;
    int n_slices_recon = (n_slices_requested - 1) + (n_slices_block - (n_slices_requested - 1) % n_slices_block);
    recon_end_pos = recon_start_pos + recon_direction * (n_slices_recon - 1) * rp.coll_slicewidth;
    int n_blocks = n_slices_recon / n_slices_block;
    int array_direction = fabs(mr->table_positions[100] - mr->table_positions[0]) /
                          (mr->table_positions[100] - mr->table_positions[0]);
    int idx_slice_start = array_search(recon_start_pos, mr->table_positions, rp.n_readings, array_direction);
    int idx_slice_end = array_search(recon_end_pos, mr->table_positions, rp.n_readings, array_direction);
    mr->ri.data_begin_pos = mr->table_positions[0];
    mr->ri.data_end_pos = mr->table_positions[rp.n_readings - 1];
    float projection_padding = cg.z_rot * (cg.n_proj_ffs / 2 + cg.add_projections_ffs + 256) / cg.n_proj_ffs;
    float allowed_begin = mr->ri.data_begin_pos + array_direction * projection_padding;
    float allowed_end = mr->ri.data_end_pos - array_direction * projection_padding;
    mr->ri.allowed_begin = allowed_begin;
    mr->ri.allowed_end = allowed_end;
    if (((rp.start_pos > allowed_begin) && (rp.start_pos > allowed_end)) ||
        ((rp.start_pos < allowed_begin) && (rp.start_pos < allowed_end)))
        return 3;
    if (((rp.end_pos > allowed_begin) && (rp.end_pos > allowed_end)) ||
        ((rp.end_pos < allowed_begin) && (rp.end_pos < allowed_end)))
        return 3;
    int pull_start, pull_end, n_pull;
    pull_window(cg, n_ffs, idx_slice_start, idx_slice_end, &pull_start, &pull_end, &n_pull);
    mr->cg.table_direction = array_direction;  // :590-603
    mr->rp.end_pos = rp.end_pos;
    mr->ri.n_ffs = n_ffs;
    mr->ri.n_slices_requested = n_slices_requested;
    mr->ri.n_slices_recon = n_slices_recon;
    mr->ri.n_slices_block = n_slices_block;
    mr->ri.n_blocks = n_blocks;
    mr->ri.idx_slice_start = idx_slice_start;
    mr->ri.idx_slice_end = idx_slice_end;
    mr->ri.recon_start_pos = recon_start_pos;
    mr->ri.recon_end_pos = recon_end_pos;
    mr->ri.idx_pull_start = pull_start;
    mr->ri.idx_pull_end = pull_end;
    mr->ri.n_proj_pull = n_pull;
    return 0;
}

// update_block_info without the host re-allocation.
int oracle_update_block_info(struct recon_metadata *mr)
{
    struct recon_info ri = mr->ri;
    struct recon_params rp = mr->rp;
    struct ct_geom cg = mr->cg;
    int n_ffs = pow(2, rp.z_ffs) * pow(2, rp.phi_ffs);
    int recon_direction = fabs(rp.end_pos - rp.start_pos) / (rp.end_pos - rp.start_pos);
    if (recon_direction != 1 && recon_direction != -1) recon_direction = 1;
    float block_slice_start =
        ri.recon_start_pos + recon_direction * ri.cb.block_idx * rp.coll_slicewidth * (float)ri.n_slices_block;
    float block_slice_end =
        block_slice_start + (float)recon_direction * ((float)ri.n_slices_block - 1.0f) * rp.coll_slicewidth;
    int array_direction = fabs(mr->table_positions[100] - mr->table_positions[0]) /
                          (mr->table_positions[100] - mr->table_positions[0]);
    int idx_block_slice_start = array_search(block_slice_start, mr->table_positions, rp.n_readings, array_direction);
    int idx_block_slice_end = array_search(block_slice_end, mr->table_positions, rp.n_readings, array_direction);
    int pull_start, pull_end, n_pull;
    pull_window(cg, n_ffs, idx_block_slice_start, idx_block_slice_end, &pull_start, &pull_end, &n_pull);
    mr->ri.cb.block_slice_start = block_slice_start;
    mr->ri.cb.block_slice_end = block_slice_end;
    mr->ri.cb.idx_block_slice_start = idx_block_slice_start;
    mr->ri.cb.idx_block_slice_end = idx_block_slice_end;
    mr->ri.idx_pull_start = pull_start;
    mr->ri.idx_pull_end = pull_end;
    mr->ri.n_proj_pull = n_pull;
    mr->ri.cb.block_idx++;
    return 0;
}

int oracle_free_plan(struct recon_metadata *mr)
{
    free(mr->tube_angles);
    free(mr->table_positions);
    mr->tube_angles = nullptr;
    mr->table_positions = nullptr;
    return 0;
}

// resources/ramp.m: f = (c^2 / (2 ds)) (a r(c pi k) + (1-a)/2 r(pi c k + pi)
// + (1-a)/2 r(pi c k - pi)), r(t) = sin t / t + (cos t - 1) / t^2, r(0) = 1/2,
// for k = j - n_os, j in [0, 2 n_os); evaluated in double, stored as float.
int oracle_ramp_taps(int n_os, float ds, float c, float a, float *taps)
{
    const double PI = 3.14159265358979323846;
    auto r = [](double t) { return t == 0.0 ? 0.5 : std::sin(t) / t + (std::cos(t) - 1.0) / (t * t); };
    for (int j = 0; j < 2 * n_os; ++j) {
        double k = (double)(j - n_os);
        double v = ((double)c * c / (2.0 * ds)) *
                   (a * r(c * PI * k) + ((1.0 - a) / 2.0) * r(PI * c * k + PI) + ((1.0 - a) / 2.0) * r(PI * c * k - PI));
        taps[j] = (float)v;
    }
    return 0;
}

}  // extern "C"

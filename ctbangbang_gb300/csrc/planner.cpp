// planner.cpp -- host planner: .prm / .scanner parsing, scanner geometry,
// per-frame tables, 32-slice blocks and pull windows, filter taps.
//
// Every integer this file produces must equal the reference's (src/setup.cu),
// so each formula is evaluated with the same C++ types and operation order as
// there: float where the reference computes in float, double where it promotes,
// size_t/int conversions at the same points.  The file is compiled with
// -ffp-contract=off so that no platform fuses a multiply-add the reference
// performs as two roundings.
#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "ctbb_internal.h"

namespace ctbb {

static thread_local char g_last_error[1024] = {0};

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

void clear_error() { g_last_error[0] = 0; }

const char *last_error_text() { return g_last_error; }

// src/setup.cu:806-825.  The reference reads array[idx] before testing
// idx < numel; the bound is tested first here, which returns the same index.
int array_search(float key, const double *array, int numel, int search_type)
{
    int idx = 0;
    switch (search_type) {
    case -1:
        while (idx < numel && key < array[idx]) idx++;
        break;
    case 0:
        while (idx < numel && key != array[idx]) idx++;
        break;
    case 1:
        while (idx < numel && key > array[idx]) idx++;
        break;
    default:
        break;
    }
    return idx;
}

// fabs(end-start)/(end-start) converted to int; a single slice (0/0) gives 1.
int recon_direction_of(const struct recon_params &rp)
{
    float diff = rp.end_pos - rp.start_pos;
    if (diff == 0.0f || std::isnan(diff)) return 1;
    int d = (int)(std::fabs(diff) / diff);
    if (d != 1 && d != -1) d = 1;
    return d;
}

int array_direction_of(const double *tp)
{
    double diff = tp[100] - tp[0];
    if (diff == 0.0 || std::isnan(diff)) return 0;
    return (int)(std::fabs(diff) / diff);
}

// Pull window around frames [idx_a, idx_b] (either order), src/setup.cu:557-581
// and :637-661: half a turn plus add_projections_ffs on each side, rounded up to
// a multiple of n_ffs with C's truncating remainder, 256 extra frames at the
// end, and the frame count rounded up to a multiple of 128.
void pull_window(const struct ct_geom &cg, int n_ffs, int idx_a, int idx_b,
                 int *idx_pull_start, int *idx_pull_end, int *n_proj_pull)
{
    int pre_post_buffer = (int)(cg.n_proj_ffs / 2);
    int lo = idx_a, hi = idx_b;
    if (idx_a > idx_b) {
        lo = idx_b;
        hi = idx_a;
    }
    // int - int - size_t wraps through size_t and back to int in the reference;
    // two's complement makes that the plain int result.
    int s = (int)((size_t)(lo - pre_post_buffer) - cg.add_projections_ffs);
    s = (s - 1) + (n_ffs - (s - 1) % n_ffs);
    int e = (int)((size_t)(hi + pre_post_buffer) + cg.add_projections_ffs);
    e = (e - 1) + (n_ffs - (e - 1) % n_ffs);
    e += 256;
    int n = e - s;
    n = (n - 1) + (128 - (n - 1) % 128);
    e = s + n;
    *idx_pull_start = s;
    *idx_pull_end = e;
    *n_proj_pull = n;
}

BlockDims block_dims(const struct recon_metadata &mr)
{
    BlockDims d;
    d.n_proj_pull = mr.ri.n_proj_pull;
    d.n_ffs = mr.ri.n_ffs;
    d.n_proj = d.n_ffs ? d.n_proj_pull / d.n_ffs : 0;
    d.n_views = d.n_proj - 2 * mr.cg.add_projections;
    d.n_channels = mr.cg.n_channels;
    d.n_os = mr.cg.n_channels_oversampled;
    d.n_rows = mr.cg.n_rows;
    d.n_rows_raw = mr.cg.n_rows_raw;
    // src/backproject_cpu.cu:56: (size_t expression) / (size_t) -> int
    d.n_half_turns = (int)((mr.ri.n_proj_pull / mr.ri.n_ffs - 2 * mr.cg.add_projections) /
                           (mr.cg.n_proj_turn / 2));
    return d;
}

float bp_tube_start(const struct recon_metadata &mr)
{
    const struct ct_geom &cg = mr.cg;
    float frames = (float)(mr.ri.idx_pull_start + cg.add_projections_ffs);
    float a = mr.tube_angles[0] + (frames * 360.0f / (float)cg.n_proj_ffs);
    double wrapped = std::fmod((double)a, 360.0);
    return (float)(wrapped * (double)kPiBackproject / (double)180.0f);
}

}  // namespace ctbb

using namespace ctbb;

extern "C" const char *ctbb_last_error(void) { return last_error_text(); }

// --------------------------------------------------------------------------
// .prm parsing (src/parse_config.cu:40-217, src/setup.cu:108-176)
// --------------------------------------------------------------------------

namespace {

enum class Kind { Str, Int, UInt, Float };
struct PrmKey {
    const char *token;
    Kind kind;
    size_t offset;
    size_t size;
};

#define CTBB_KEY(tok, kind, field) \
    { tok, kind, offsetof(struct recon_params, field), sizeof(((struct recon_params *)0)->field) }

const PrmKey kPrmKeys[] = {
    CTBB_KEY("RawDataDir:", Kind::Str, raw_data_dir),
    CTBB_KEY("RawDataFile:", Kind::Str, raw_data_file),
    CTBB_KEY("OutputDir:", Kind::Str, output_dir),
    CTBB_KEY("OutputFile:", Kind::Str, output_file),
    CTBB_KEY("Nrows:", Kind::Int, n_rows),
    CTBB_KEY("CollSlicewidth:", Kind::Float, coll_slicewidth),
    CTBB_KEY("StartPos:", Kind::Float, start_pos),
    CTBB_KEY("EndPos:", Kind::Float, end_pos),
    CTBB_KEY("TableFeed:", Kind::Float, pitch_value),
    CTBB_KEY("PitchValue:", Kind::Float, pitch_value),
    CTBB_KEY("SliceThickness:", Kind::Float, slice_thickness),
    CTBB_KEY("AcqFOV:", Kind::Float, acq_fov),
    CTBB_KEY("ReconFOV:", Kind::Float, recon_fov),
    CTBB_KEY("ReconKernel:", Kind::Int, recon_kernel),
    CTBB_KEY("Readings:", Kind::Int, n_readings),
    CTBB_KEY("Xorigin:", Kind::Float, x_origin),
    CTBB_KEY("Yorigin:", Kind::Float, y_origin),
    CTBB_KEY("Zffs:", Kind::Int, z_ffs),
    CTBB_KEY("Phiffs:", Kind::Int, phi_ffs),
    CTBB_KEY("Scanner:", Kind::Str, scanner),
    CTBB_KEY("FileType:", Kind::Int, file_type),
    CTBB_KEY("FileSubType:", Kind::Int, file_subtype),
    CTBB_KEY("RawOffset:", Kind::Int, raw_data_offset),
    CTBB_KEY("Nx:", Kind::UInt, nx),
    CTBB_KEY("Ny:", Kind::UInt, ny),
    CTBB_KEY("TubeStartAngle:", Kind::Float, tube_start_angle),
    CTBB_KEY("AdaptiveFiltration:", Kind::Float, adaptive_filtration_s),
    CTBB_KEY("NSlices:", Kind::Int, n_slices),
    CTBB_KEY("TableDir:", Kind::Str, table_dir_str),
    CTBB_KEY("TableDirInt:", Kind::Int, table_dir),
};
#undef CTBB_KEY

void assign_key(struct recon_params *rp, const PrmKey &k, const char *value)
{
    char *base = reinterpret_cast<char *>(rp) + k.offset;
    switch (k.kind) {
    case Kind::Str: {
        char buf[8192];
        if (sscanf(value, "%8191s", buf) == 1) {
            strncpy(base, buf, k.size - 1);
            base[k.size - 1] = 0;
        }
        break;
    }
    case Kind::Int: sscanf(value, "%d", reinterpret_cast<int *>(base)); break;
    case Kind::UInt: sscanf(value, "%u", reinterpret_cast<unsigned *>(base)); break;
    case Kind::Float: sscanf(value, "%f", reinterpret_cast<float *>(base)); break;
    }
}

}  // namespace

extern "C" int ctbb_configure_recon_params(const char *prm_path, struct recon_params *out)
{
    clear_error();
    if (!prm_path || !out) {
        set_error("ctbb_configure_recon_params: null argument");
        return CTBB_ERR_ARGUMENT;
    }
    FILE *f = fopen(prm_path, "r");
    if (!f) {
        set_error("parameter file %s not found", prm_path);
        return CTBB_ERR_IO;
    }
    struct recon_params rp;
    memset(&rp, 0, sizeof(rp));
    char line[1024];
    while (fgets(line, sizeof(line), f)) {
        char *pct = strchr(line, '%');  // comments start at '%'
        if (pct) *pct = 0;
        char *save = nullptr;
        char *tok = strtok_r(line, " \t\r\n", &save);
        if (!tok) continue;
        char *val = strtok_r(nullptr, " \t\r\n", &save);
        for (const PrmKey &k : kPrmKeys) {
            if (strcmp(tok, k.token) == 0 && val) assign_key(&rp, k, val);
        }
    }
    fclose(f);

    if (strcmp(rp.table_dir_str, "") != 0) {
        if (strcmp(rp.table_dir_str, "out") == 0)
            rp.table_dir = 1;
        else if (strcmp(rp.table_dir_str, "in") == 0)
            rp.table_dir = -1;
        else
            rp.table_dir = 1;  // the reference warns and defaults to "out"
    }
    const char *missing = nullptr;
    if (rp.n_rows == 0) missing = "Nrows";
    else if (rp.coll_slicewidth == 0) missing = "CollSlicewidth";
    else if (rp.slice_thickness == 0) missing = "SliceThickness";
    else if (rp.pitch_value == 0) missing = "PitchValue";
    else if (rp.acq_fov == 0) missing = "AcqFOV";
    else if (rp.recon_fov == 0) missing = "ReconFOV";
    else if (rp.n_readings == 0) missing = "Readings";
    else if (rp.nx == 0) missing = "Nx";
    else if (rp.ny == 0) missing = "Ny";
    if (rp.file_type == 0 && rp.table_dir == 0) rp.table_dir = 1;
    *out = rp;
    if (missing) {
        set_error("%s was not properly set in configuration", missing);
        return CTBB_ERR_CONFIG;
    }
    // Values the reference takes as they come and that would only fail later
    // (or not at all) in planning and reconstruction: rejected here.
    const struct {
        const char *name;
        float v;
        bool positive;
    } floats[] = {
        {"CollSlicewidth", rp.coll_slicewidth, true}, {"SliceThickness", rp.slice_thickness, true},
        {"AcqFOV", rp.acq_fov, true},                  {"ReconFOV", rp.recon_fov, true},
        {"PitchValue", rp.pitch_value, false},         {"StartPos", rp.start_pos, false},
        {"EndPos", rp.end_pos, false},                 {"Xorigin", rp.x_origin, false},
        {"Yorigin", rp.y_origin, false},               {"TubeStartAngle", rp.tube_start_angle, false},
        {"AdaptiveFiltration", rp.adaptive_filtration_s, false},
    };
    for (const auto &f : floats) {
        if (!std::isfinite(f.v) || (f.positive && !(f.v > 0.0f))) {
            set_error("%s: %g is not a %snumber", f.name, (double)f.v, f.positive ? "positive finite " : "finite ");
            return CTBB_ERR_CONFIG;
        }
    }
    const unsigned kMaxSide = 16384;
    if (rp.nx > kMaxSide || rp.ny > kMaxSide) {
        set_error("Nx/Ny %u x %u: each side must be 1..%u", rp.nx, rp.ny, kMaxSide);
        return CTBB_ERR_CONFIG;
    }
    if (rp.n_rows < 0 || rp.n_readings < 0 || rp.n_slices < 0) {
        set_error("Nrows %d, Readings %d, NSlices %d: negative", rp.n_rows, rp.n_readings, rp.n_slices);
        return CTBB_ERR_CONFIG;
    }
    if ((rp.z_ffs != 0 && rp.z_ffs != 1) || (rp.phi_ffs != 0 && rp.phi_ffs != 1)) {
        set_error("Zffs %d / Phiffs %d: each must be 0 or 1", rp.z_ffs, rp.phi_ffs);
        return CTBB_ERR_CONFIG;
    }
    return CTBB_OK;
}

// --------------------------------------------------------------------------
// Scanner geometry (src/setup.cu:178-383)
// --------------------------------------------------------------------------

namespace {

bool read_scanner_file(FILE *f, struct ct_geom *cg)
{
    std::vector<char> buf;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    rewind(f);
    if (n < 0) return false;
    buf.resize((size_t)n + 1, 0);
    size_t got = fread(buf.data(), 1, (size_t)n, f);
    buf[got] = 0;
    // Tokens are separated by blanks, newlines and '%' (src/setup.cu:232,280);
    // a key token is followed by its value token.
    char *save = nullptr;
    char *tok = strtok_r(buf.data(), " \t\n%", &save);
    while (tok) {
        auto next = [&]() { return strtok_r(nullptr, " \t\n%", &save); };
        char *val = nullptr;
        if (strcmp(tok, "RSrcToIso:") == 0) { if ((val = next())) sscanf(val, "%f", &cg->r_f); }
        else if (strcmp(tok, "RSrcToDet:") == 0) { if ((val = next())) sscanf(val, "%f", &cg->src_to_det); }
        else if (strcmp(tok, "AnodeAngle:") == 0) { if ((val = next())) sscanf(val, "%f", &cg->anode_angle); }
        else if (strcmp(tok, "FanAngleInc:") == 0) { if ((val = next())) sscanf(val, "%f", &cg->fan_angle_increment); }
        else if (strcmp(tok, "ThetaCone:") == 0) { if ((val = next())) sscanf(val, "%f", &cg->theta_cone); }
        else if (strcmp(tok, "CentralChannel:") == 0) { if ((val = next())) sscanf(val, "%f", &cg->central_channel); }
        else if (strcmp(tok, "NProjTurn:") == 0) { if ((val = next())) sscanf(val, "%zu", &cg->n_proj_turn); }
        else if (strcmp(tok, "NChannels:") == 0) { if ((val = next())) sscanf(val, "%zu", &cg->n_channels); }
        else if (strcmp(tok, "ReverseRowInterleave:") == 0) { if ((val = next())) sscanf(val, "%i", &cg->reverse_row_interleave); }
        else if (strcmp(tok, "ReverseChanInterleave:") == 0) { if ((val = next())) sscanf(val, "%i", &cg->reverse_channel_interleave); }
        tok = next();
    }
    return true;
}

// Sizes derived from the detector and the .prm (identical for every scanner
// source, src/setup.cu:291-297 and the three built-in cases).
void finish_geometry(struct ct_geom *cg, const struct recon_params &rp)
{
    cg->n_proj_ffs = (size_t)(cg->n_proj_turn * pow(2, rp.phi_ffs) * pow(2, rp.z_ffs));
    cg->n_channels_oversampled = 2 * cg->n_channels;
    cg->n_rows = (unsigned int)rp.n_rows;
    cg->n_rows_raw = (unsigned int)(rp.n_rows / pow(2, rp.z_ffs));
    cg->z_rot = rp.pitch_value;
    float fan_half = cg->fan_angle_increment * (float)cg->n_channels / 2;
    float view_step = 2.0f * kPiRebin / (float)cg->n_proj_turn;
    cg->add_projections = (size_t)(fan_half / view_step + 10);
    cg->add_projections_ffs = (size_t)(cg->add_projections * pow(2, rp.z_ffs) * pow(2, rp.phi_ffs));
}

}  // namespace

extern "C" int ctbb_configure_ct_geom(struct recon_metadata *mr)
{
    clear_error();
    if (!mr) {
        set_error("ctbb_configure_ct_geom: null metadata");
        return CTBB_ERR_ARGUMENT;
    }
    struct recon_params &rp = mr->rp;
    struct ct_geom cg;
    memset(&cg, 0, sizeof(cg));
    cg.table_direction = rp.table_dir;

    int scanner = -1;
    FILE *f = fopen(rp.scanner, "r");
    if (!f) {
        char path[4096 + 4351 + 64];
        snprintf(path, sizeof(path), "%s/resources/scanners/%s", mr->install_dir, rp.scanner);
        f = fopen(path, "r");
    }
    if (!f) {
        scanner = atoi(rp.scanner);
        if (scanner < 0 || scanner > 2 || (scanner == 0 && strlen(rp.scanner) != 1)) {
            set_error("could not parse selected scanner '%s'", rp.scanner);
            return CTBB_ERR_CONFIG;
        }
        if (scanner == 1) rp.file_subtype = 1;
        if (scanner == 2) rp.file_subtype = 2;
    }

    if (scanner == -1) {
        bool ok = read_scanner_file(f, &cg);
        fclose(f);
        if (!ok) {
            set_error("could not read scanner file '%s'", rp.scanner);
            return CTBB_ERR_IO;
        }
    } else {
        // Built-in scanners, src/setup.cu:300-372 (the reference's constants).
        switch (scanner) {
        case 0:  // simulated Sensation 64
            cg.r_f = 570.0f;
            cg.src_to_det = 1040.0f;
            cg.anode_angle = 7.0f * kPiRebin / 180.0f;
            cg.fan_angle_increment = 1.4083f / cg.src_to_det;
            cg.theta_cone = 2.0f * std::atan(7.5f * 1.3684f / cg.src_to_det);
            cg.central_channel = 335.25f;
            cg.n_proj_turn = 1160;
            cg.n_channels = 672;
            break;
        case 1:  // Definition AS
            cg.r_f = 595.0f;
            cg.src_to_det = 1085.6f;
            cg.anode_angle = 7.0f * kPiRebin / 180.0f;
            cg.fan_angle_increment = 0.067864f * kPiRebin / 180.0f;
            cg.theta_cone = 2.0f * std::atan(7.5f * 1.2f / cg.r_f);
            cg.central_channel = 366.25f;
            cg.n_proj_turn = 1152;
            cg.n_channels = 736;
            break;
        default:  // Sensation 64
            cg.r_f = 570.0f;
            cg.src_to_det = 1040.0f;
            cg.anode_angle = 7.0f * kPiRebin / 180.0f;
            cg.fan_angle_increment = 0.07758621f * kPiRebin / 180.0f;
            cg.theta_cone = 2.0f * std::atan(7.5f * 1.2f / cg.r_f);
            cg.central_channel = 334.25f;
            cg.n_proj_turn = 1160;
            cg.n_channels = 672;
            break;
        }
    }
    if (cg.n_proj_turn == 0 || cg.n_channels == 0) {
        set_error("scanner geometry lacks NProjTurn or NChannels");
        return CTBB_ERR_CONFIG;
    }
    finish_geometry(&cg, rp);
    cg.acq_fov = rp.acq_fov;
    if (rp.phi_ffs == 1) cg.central_channel = std::floor(cg.central_channel) + 0.375f;
    mr->cg = cg;
    return CTBB_OK;
}

// --------------------------------------------------------------------------
// Reconstruction plan (src/setup.cu:385-679)
// --------------------------------------------------------------------------

namespace {

int alloc_block_arrays(struct recon_metadata *mr, int n_proj_pull)
{
    const struct ct_geom &cg = mr->cg;
    int n_ffs = (int)mr->ri.n_ffs;
    size_t n_raw = cg.n_channels * cg.n_rows_raw * (size_t)n_proj_pull;
    size_t n_rebin = cg.n_channels_oversampled * cg.n_rows *
                     ((size_t)n_proj_pull - 2 * cg.add_projections_ffs) / (size_t)n_ffs;
    mr->ctd.raw = (float *)calloc(n_raw, sizeof(float));
    mr->ctd.rebin = (float *)calloc(n_rebin, sizeof(float));
    if (!mr->ctd.raw || !mr->ctd.rebin) {
        set_error("host allocation of raw/rebin (%zu + %zu floats) failed", n_raw, n_rebin);
        return CTBB_ERR_ALLOC;
    }
    return CTBB_OK;
}

}  // namespace

extern "C" int ctbb_configure_reconstruction(struct recon_metadata *mr)
{
    clear_error();
    if (!mr) {
        set_error("ctbb_configure_reconstruction: null metadata");
        return CTBB_ERR_ARGUMENT;
    }
    const struct ct_geom cg = mr->cg;
    struct recon_params rp = mr->rp;
    if (rp.n_readings <= 1000) {
        set_error("Readings must exceed 1000 (table direction is taken from frame 1000)");
        return CTBB_ERR_CONFIG;
    }
    if (rp.file_type != 0) {
        set_error("FileType %d: only FileType 0 (float32 binary frames) is supported",
                  rp.file_type);
        return CTBB_ERR_CONFIG;
    }
    free(mr->tube_angles);
    free(mr->table_positions);
    mr->tube_angles = (float *)calloc((size_t)rp.n_readings, sizeof(float));
    mr->table_positions = (double *)calloc((size_t)rp.n_readings, sizeof(double));
    if (!mr->tube_angles || !mr->table_positions) {
        set_error("host allocation of frame tables failed");
        return CTBB_ERR_ALLOC;
    }
    // FileType 0 tables, src/setup.cu:405-415.
    for (int i = 0; i < rp.n_readings; i++) {
        mr->tube_angles[i] =
            std::fmod(((360.0f / (float)cg.n_proj_ffs) * (float)i + rp.tube_start_angle), 360.0f);
        if (cg.table_direction == -1)
            mr->table_positions[i] =
                ((float)rp.n_readings / (float)cg.n_proj_ffs) * cg.z_rot -
                (float)i * cg.z_rot / (float)cg.n_proj_ffs;
        else
            mr->table_positions[i] = 0.0f + (float)i * cg.z_rot / (float)cg.n_proj_ffs;
    }

    int n_ffs = (int)(pow(2, rp.z_ffs) * pow(2, rp.phi_ffs));
    int n_slices_block = kBlockSlices;
    int recon_direction = recon_direction_of(rp);
    if (rp.n_slices != 0) rp.end_pos = rp.start_pos + (float)(rp.n_slices - 1) * rp.slice_thickness;

    float recon_start_pos = rp.start_pos - (float)recon_direction * rp.slice_thickness;
    float recon_end_pos = rp.end_pos + (float)recon_direction * rp.slice_thickness;
    int n_slices_requested =
        (int)(std::floor(std::fabs(recon_end_pos - recon_start_pos) / rp.coll_slicewidth) + 1.0f);
    int n_slices_recon =
        (n_slices_requested - 1) + (n_slices_block - (n_slices_requested - 1) % n_slices_block);
    recon_end_pos = recon_start_pos +
                    (float)(recon_direction * (n_slices_recon - 1)) * rp.coll_slicewidth;
    int n_blocks = n_slices_recon / n_slices_block;

    int array_direction = array_direction_of(mr->table_positions);
    int idx_slice_start = array_search(recon_start_pos, mr->table_positions, rp.n_readings,
                                       array_direction);
    int idx_slice_end =
        array_search(recon_end_pos, mr->table_positions, rp.n_readings, array_direction);

    mr->ri.data_begin_pos = (float)mr->table_positions[0];
    mr->ri.data_end_pos = (float)mr->table_positions[rp.n_readings - 1];
    float projection_padding =
        cg.z_rot * (float)(cg.n_proj_ffs / 2 + cg.add_projections_ffs + 256) / (float)cg.n_proj_ffs;
    float allowed_begin = mr->ri.data_begin_pos + (float)array_direction * projection_padding;
    float allowed_end = mr->ri.data_end_pos - (float)array_direction * projection_padding;
    mr->ri.allowed_begin = allowed_begin;
    mr->ri.allowed_end = allowed_end;

    auto outside = [&](float p) {
        return ((p > allowed_begin) && (p > allowed_end)) || ((p < allowed_begin) && (p < allowed_end));
    };
    if (outside(rp.start_pos) || outside(rp.end_pos)) {
        set_error("requested reconstruction is outside of allowed data range: %.2f to %.2f",
                  allowed_begin, allowed_end);
        return CTBB_ERR_RANGE;
    }

    int idx_pull_start, idx_pull_end, n_proj_pull;
    pull_window(cg, n_ffs, idx_slice_start, idx_slice_end, &idx_pull_start, &idx_pull_end,
                &n_proj_pull);

    mr->cg.table_direction = array_direction;
    mr->rp.end_pos = rp.end_pos;
    mr->ri.n_ffs = (size_t)n_ffs;
    mr->ri.n_slices_requested = (size_t)n_slices_requested;
    mr->ri.n_slices_recon = (size_t)n_slices_recon;
    mr->ri.n_slices_block = (size_t)n_slices_block;
    mr->ri.n_blocks = (size_t)n_blocks;
    mr->ri.idx_slice_start = (size_t)idx_slice_start;
    mr->ri.idx_slice_end = (size_t)idx_slice_end;
    mr->ri.recon_start_pos = recon_start_pos;
    mr->ri.recon_end_pos = recon_end_pos;
    mr->ri.idx_pull_start = (size_t)idx_pull_start;
    mr->ri.idx_pull_end = (size_t)idx_pull_end;
    mr->ri.n_proj_pull = (size_t)n_proj_pull;

    int st = alloc_block_arrays(mr, n_proj_pull);
    if (st) return st;
    mr->ctd.image = (float *)calloc((size_t)rp.nx * rp.ny * (size_t)n_slices_recon, sizeof(float));
    if (!mr->ctd.image) {
        set_error("host allocation of the image stack failed");
        return CTBB_ERR_ALLOC;
    }
    return CTBB_OK;
}

namespace ctbb {

// Block plan of src/setup.cu:605-679 without the host re-allocation: fills the
// block fields of *ri for block mr.ri.cb.block_idx and advances block_idx.
int plan_next_block(const struct recon_metadata &mr, struct recon_info *ri_out)
{
    const struct recon_info ri = mr.ri;
    const struct recon_params rp = mr.rp;
    const struct ct_geom cg = mr.cg;
    if (!mr.table_positions) {
        set_error("block plan: metadata not configured");
        return CTBB_ERR_STATE;
    }
    int n_ffs = (int)(pow(2, rp.z_ffs) * pow(2, rp.phi_ffs));
    int recon_direction = recon_direction_of(rp);
    float block_slice_start = ri.recon_start_pos + (float)(recon_direction * ri.cb.block_idx) *
                                                       rp.coll_slicewidth * (float)ri.n_slices_block;
    float block_slice_end = block_slice_start + (float)recon_direction *
                                                    ((float)ri.n_slices_block - 1.0f) *
                                                    rp.coll_slicewidth;
    int array_direction = array_direction_of(mr.table_positions);
    int idx_block_slice_start =
        array_search(block_slice_start, mr.table_positions, rp.n_readings, array_direction);
    int idx_block_slice_end =
        array_search(block_slice_end, mr.table_positions, rp.n_readings, array_direction);

    int idx_pull_start, idx_pull_end, n_proj_pull;
    pull_window(cg, n_ffs, idx_block_slice_start, idx_block_slice_end, &idx_pull_start,
                &idx_pull_end, &n_proj_pull);

    *ri_out = ri;
    ri_out->cb.block_slice_start = block_slice_start;
    ri_out->cb.block_slice_end = block_slice_end;
    ri_out->cb.idx_block_slice_start = idx_block_slice_start;
    ri_out->cb.idx_block_slice_end = idx_block_slice_end;
    ri_out->idx_pull_start = (size_t)idx_pull_start;
    ri_out->idx_pull_end = (size_t)idx_pull_end;
    ri_out->n_proj_pull = (size_t)n_proj_pull;
    ri_out->cb.block_idx++;
    return CTBB_OK;
}

}  // namespace ctbb

extern "C" int ctbb_update_block_info(struct recon_metadata *mr)
{
    clear_error();
    if (!mr || !mr->table_positions) {
        set_error("ctbb_update_block_info: metadata not configured");
        return CTBB_ERR_STATE;
    }
    free(mr->ctd.raw);
    free(mr->ctd.rebin);
    mr->ctd.raw = mr->ctd.rebin = nullptr;
    struct recon_info ri;
    int st = plan_next_block(*mr, &ri);
    if (st) return st;
    mr->ri = ri;
    return alloc_block_arrays(mr, (int)ri.n_proj_pull);
}

extern "C" int ctbb_extract_projections(struct recon_metadata *mr)
{
    clear_error();
    if (!mr || !mr->ctd.raw) {
        set_error("ctbb_extract_projections: metadata not configured");
        return CTBB_ERR_STATE;
    }
    char path[4096 + 255 + 2];
    snprintf(path, sizeof(path), "%s/%s", mr->rp.raw_data_dir, mr->rp.raw_data_file);
    FILE *f = fopen(path, "rb");
    if (!f) {
        set_error("raw data file %s not found", path);
        return CTBB_ERR_IO;
    }
    size_t frame = mr->cg.n_channels * mr->cg.n_rows_raw;
    for (size_t i = 0; i < mr->ri.n_proj_pull; i++) {
        float *dst = mr->ctd.raw + i * frame;
        memset(dst, 0, frame * sizeof(float));
        // idx_pull_start may be "negative" (wrapped size_t): such frames read as zeros
        long long idx = (long long)(int)(mr->ri.idx_pull_start + i);
        if (idx < 0) continue;
        long long pos = (long long)mr->rp.raw_data_offset + idx * (long long)(frame * sizeof(float));
        if (fseeko(f, (off_t)pos, SEEK_SET) != 0) continue;
        size_t got = fread(dst, sizeof(float), frame, f);
        (void)got;  // frames past the end of the file stay zero
    }
    fclose(f);
    return CTBB_OK;
}

extern "C" int ctbb_n_slices_final(const struct recon_metadata *mr)
{
    if (!mr || mr->rp.slice_thickness == 0) return 0;
    return (int)(std::floor(std::fabs(mr->rp.end_pos - mr->rp.start_pos) / mr->rp.slice_thickness) +
                 1.0f);
}

extern "C" int ctbb_finish_and_cleanup(struct recon_metadata *mr)
{
    clear_error();
    if (!mr) {
        set_error("ctbb_finish_and_cleanup: null metadata");
        return CTBB_ERR_ARGUMENT;
    }
    int status = CTBB_OK;
    if (mr->ctd.final_image_stack) {
        int n_final = ctbb_n_slices_final(mr);
        char path[4096 + 255 + 2];
        snprintf(path, sizeof(path), "%s/%s", mr->rp.output_dir, mr->rp.output_file);
        FILE *f = fopen(path, "wb");
        if (!f) {
            set_error("cannot write output file %s", path);
            status = CTBB_ERR_IO;
        } else {
            size_t n = (size_t)mr->rp.nx * mr->rp.ny * (size_t)n_final;
            if (fwrite(mr->ctd.final_image_stack, sizeof(float), n, f) != n) {
                set_error("short write to %s", path);
                status = CTBB_ERR_IO;
            }
            fclose(f);
        }
    }
    free(mr->ctd.rebin);
    free(mr->ctd.image);
    free(mr->ctd.raw);
    free(mr->ctd.final_image_stack);
    free(mr->tube_angles);
    free(mr->table_positions);
    mr->ctd.rebin = mr->ctd.image = mr->ctd.raw = mr->ctd.final_image_stack = nullptr;
    mr->tube_angles = nullptr;
    mr->table_positions = nullptr;
    return status;
}

// --------------------------------------------------------------------------
// Reconstruction kernel taps (src/rebin_filter.cu:922-959, resources/ramp.m)
// --------------------------------------------------------------------------

extern "C" int ctbb_ramp_filter_taps(int n_os, float ds, float c, float a, float *taps)
{
    if (n_os <= 0 || !taps || !(ds > 0)) {
        set_error("ctbb_ramp_filter_taps: bad argument");
        return CTBB_ERR_ARGUMENT;
    }
    const double pi = 3.14159265358979323846;
    auto r = [](double t) {
        if (t == 0.0) return 0.5;
        return std::sin(t) / t + (std::cos(t) - 1.0) / (t * t);
    };
    for (int j = 0; j < 2 * n_os; ++j) {
        double k = (double)(j - n_os);
        double t = c * pi * k;
        double v = (double)c * c / (2.0 * ds) *
                   (a * r(t) + (1.0 - a) / 2.0 * r(t + pi) + (1.0 - a) / 2.0 * r(t - pi));
        taps[j] = (float)v;
    }
    return CTBB_OK;
}

extern "C" int ctbb_load_filter(const struct recon_metadata *mr, float *taps)
{
    clear_error();
    if (!mr || !taps) {
        set_error("ctbb_load_filter: null argument");
        return CTBB_ERR_ARGUMENT;
    }
    const struct ct_geom &cg = mr->cg;
    const char *name = nullptr;
    switch (mr->rp.recon_kernel) {
    case -100: name = "ramp"; break;
    case -1: name = "exp"; break;
    case 1: name = "smooth"; break;
    case 2: name = "medium"; break;
    case 3: name = "sharp"; break;
    default: break;
    }
    char path[4096 + 128];
    if (name)
        snprintf(path, sizeof(path), "%s/resources/filters/f_%zu_%s.txt", mr->install_dir,
                 cg.n_channels, name);
    else
        snprintf(path, sizeof(path), "%s/resources/filters/f_%zu_b%i.txt", mr->install_dir,
                 cg.n_channels, mr->rp.recon_kernel);
    size_t n = 2 * cg.n_channels_oversampled;
    FILE *f = fopen(path, "rb");
    if (!f) {
        if (mr->rp.recon_kernel == -100) {
            // f_<N>_ramp is not shipped with the reference; generate the plain
            // ramp (c = 1, a = 1, ds = r_f sin(fan_angle_increment / 2)).
            float ds = (float)(cg.r_f * std::sin(cg.fan_angle_increment / 2.0));
            return ctbb_ramp_filter_taps((int)cg.n_channels_oversampled, ds, 1.0f, 1.0f, taps);
        }
        set_error("filter file %s not found", path);
        return CTBB_ERR_IO;
    }
    size_t got = fread(taps, sizeof(float), n, f);
    fclose(f);
    if (got != n) {
        set_error("filter file %s holds %zu taps, %zu expected", path, got, n);
        return CTBB_ERR_IO;
    }
    return CTBB_OK;
}

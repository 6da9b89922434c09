// abi.cu -- the library's C ABI: the work-buffer context (bound to one
// device), the device stages, the block-loop and whole-scan reconstruction
// paths (device buffers, host buffers, the raw file) and the drop-in module
// functions with the reference's semantics (host buffers in, host buffers
// out, d_rebin handed from rebin_filter to backproject).
#include <cuda_runtime.h>
#include <fcntl.h>
#include <unistd.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <new>
#include <condition_variable>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <thread>
#include <vector>

#include "adaptive_filter.h"
#include "backproject.h"
#include "ctbb_internal.h"
#include "cuda_util.cuh"
#include "finalize.h"
#include "ramp_filter.h"
#include "ramp_tc.h"
#include "rebin.h"

namespace ctbb {

namespace {

// Stages timed by ctbb_profile_*: adaptive filter, rebin, ramp filter,
// backprojection, finalize.
constexpr int kProfileStages = 5;

// Grow-only device buffer.
struct DeviceBuffer {
    void *ptr = nullptr;
    size_t bytes = 0;
    int ensure(size_t need)
    {
        if (need <= bytes && ptr) return CTBB_OK;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&ptr, need ? need : 16);
        if (e != cudaSuccess) {
            set_error("cudaMalloc of %zu bytes failed: %s", need, cudaGetErrorString(e));
            ptr = nullptr;
            return CTBB_ERR_ALLOC;
        }
        bytes = need;
        return CTBB_OK;
    }
    void release()
    {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template <class T>
    T *as() const { return reinterpret_cast<T *>(ptr); }
};

struct Context {
    std::mutex mu;
    cudaStream_t stream = nullptr;
    std::atomic<uint64_t> launches{0};
    // stage work buffers
    DeviceBuffer raw_in, raw_filt, rebin, block, image, final_stack, scratch;
    // tables
    DeviceBuffer bp_views, bp_theta, bp_zpos, fin_offsets, fin_slices, fin_weights;
    DeviceBuffer bp_partial;  // the backprojector's partial image sums (angle chunks)
    // whole-scan paths: one block window filtered with its own statistics,
    // and per frame of each block window whether that can differ from the union
    DeviceBuffer edge_raw, dirty;
    DeviceRebinTables rebin_tables;
    RampFilterPlan ramp;
    RampTcPlan ramp_tc;
    DeviceBuffer tc_work;
    // whole-scan row storage: 0 float32 rows, 1 FP16 footprint quads + per-view
    // scales written by the tensor-core ramp filter (quads, qscale)
    int storage = 0;
    DeviceBuffer quads, qscale;
    // every block's backprojector tables of a prepared whole scan
    DeviceBuffer bp_tables;
    // time the backprojector's launch shapes once per geometry class
    bool autotune = false;
    void *our_d_rebin = nullptr;  // last d_rebin handed out by the drop-in rebin_filter
    int sms = 0;
    std::atomic<int> device{-1};  // the device the work buffers live on (-1: none yet)
    // host-buffer whole-scan path: second window buffer and a copy stream
    DeviceBuffer raw_in2;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copied[2] = {nullptr, nullptr}, consumed[2] = {nullptr, nullptr};
    // streamed whole-scan path: the preparation (adaptive filter, rebin, ramp
    // filter, edge patches) on a stream of its own, at a higher priority than
    // the backprojections it feeds; prep_ready orders a block's backprojection
    // after its rows
    cudaStream_t prep_stream = nullptr;
    cudaEvent_t prep_ready = nullptr;
    std::vector<cudaEvent_t> chunk_copied;  // whole-scan host path: one per chunk
    // streamed whole-scan path: a block's edge-frame flags read back into
    // pinned memory, flags_ready recorded behind the copy
    unsigned char *flags_host = nullptr;
    size_t flags_host_bytes = 0;
    cudaEvent_t flags_ready = nullptr;
    // whole-scan file path: two pinned staging buffers and their reuse events
    void *stage[2] = {nullptr, nullptr};
    size_t stage_bytes = 0;
    cudaEvent_t stage_free[2] = {nullptr, nullptr};
    // per-stage CUDA-event timing (ctbb_profile_*)
    bool profiling = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> open_events[kProfileStages];
    std::vector<cudaEvent_t> event_pool;
    double stage_ms[kProfileStages] = {0};
    uint64_t stage_launches[kProfileStages] = {0};
};

Context &ctx()
{
    // static storage, constructed on first use without heap allocation; its
    // destructor makes no CUDA calls (device buffers are released explicitly)
    static Context c;
    return c;
}

cudaEvent_t pooled_event(Context &c)
{
    if (!c.event_pool.empty()) {
        cudaEvent_t e = c.event_pool.back();
        c.event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Brackets the launches of one stage with events on the library stream while
// profiling is on (the events add no synchronisation).
struct StageScope {
    Context &c;
    int stage;
    cudaEvent_t start = nullptr;
    StageScope(Context &cx, int st) : c(cx), stage(st)
    {
        if (c.profiling) {
            start = pooled_event(c);
            cudaEventRecord(start, c.stream);
        }
    }
    ~StageScope()
    {
        if (start) {
            cudaEvent_t stop = pooled_event(c);
            cudaEventRecord(stop, c.stream);
            c.open_events[stage].push_back({start, stop});
        }
    }
};

template <class T>
int upload(DeviceBuffer &buf, const std::vector<T> &v, cudaStream_t s)
{
    CTBB_TRY(buf.ensure(v.size() * sizeof(T)));
    if (!v.empty())
        CTBB_CUDA_TRY(cudaMemcpyAsync(buf.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return CTBB_OK;
}

int check_mr(const struct recon_metadata *mr)
{
    if (!mr) {
        set_error("null recon_metadata");
        return CTBB_ERR_ARGUMENT;
    }
    if (mr->ri.n_ffs == 0 || mr->ri.n_proj_pull == 0 || mr->cg.n_channels == 0 || mr->cg.n_rows == 0) {
        set_error("recon_metadata is not planned (n_ffs / n_proj_pull / geometry unset)");
        return CTBB_ERR_STATE;
    }
    return CTBB_OK;
}

// Chunks the whole-scan host path copies the union window in.
int scan_chunks()
{
    static int v = [] {
        const char *e = getenv("CTBB_SCAN_CHUNKS");
        int n = e ? atoi(e) : 8;
        return n < 1 ? 1 : (n > 64 ? 64 : n);
    }();
    return v;
}

// Default voxels-per-thread of the backprojector along z.
constexpr int kBackprojectZpt = 8;

int bp_zpt()
{
    static int v = [] {
        const char *e = getenv("CTBB_BP_ZPT");
        int z = e ? atoi(e) : kBackprojectZpt;
        return (z == 4 || z == 8 || z == 16 || z == 32) ? z : kBackprojectZpt;
    }();
    return v;
}

}  // namespace

cudaStream_t current_stream() { return ctx().stream; }

int num_sms()
{
    Context &c = ctx();
    if (!c.sms) {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        c.sms = n > 0 ? n : 1;
    }
    return c.sms;
}

void count_launch(uint64_t n) { ctx().launches += n; }

int require_device(Context &c)
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        set_error("no CUDA device available (%s); this library has no CPU path",
                  e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
        return CTBB_ERR_NO_DEVICE;
    }
    // the work buffers, tables and streams belong to the device of the first
    // call; another device must not reach them
    int dev = 0;
    CTBB_CUDA_TRY(cudaGetDevice(&dev));
    int bound = -1;
    if (!c.device.compare_exchange_strong(bound, dev) && bound != dev) {
        set_error("the library's work buffers live on device %d, the current device is %d: call "
                  "ctbb_release_workspace() before switching devices", bound, dev);
        return CTBB_ERR_STATE;
    }
    return CTBB_OK;
}

// A usable CUDA device, without binding the library-wide context to it (the
// no-allocation filter holds no buffers of that context).
int require_device()
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        set_error("no CUDA device available (%s); this library has no CPU path",
                  e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
        return CTBB_ERR_NO_DEVICE;
    }
    return CTBB_OK;
}

// The adaptive filter on the library-wide stream with the caller's scratch,
// serialised with the other entry points and counted by the stage profile.
int run_adaptive_filter_with(const struct recon_metadata &mr, const float *d_in, float *d_out, float *d_scratch)
{
    Context &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    StageScope scope(c, 0);
    return launch_adaptive_filter(mr, d_in, d_out, d_scratch, c.stream);
}

// ---- stage implementations (device pointers, stream-ordered) --------------

static int do_adaptive(Context &c, const struct recon_metadata &mr, const float *d_in, float *d_out)
{
    size_t n = adaptive_filter_scratch_floats(mr.ri.n_proj_pull);
    CTBB_TRY(c.scratch.ensure(n * sizeof(float)));
    StageScope scope(c, 0);
    return launch_adaptive_filter(mr, d_in, d_out, c.scratch.as<float>(), c.stream);
}

static int do_rebin(Context &c, const struct recon_metadata &mr, const float *d_raw, float *d_rebin)
{
    RebinTables t;
    CTBB_TRY(build_rebin_tables(mr, &t));
    CTBB_TRY(upload_rebin_tables(t, &c.rebin_tables, c.stream));
    StageScope scope(c, 1);
    return launch_rebin(t, c.rebin_tables, d_raw, d_rebin, c.stream);
}

static int do_filter(Context &c, const struct recon_metadata &mr, float *d_rebin)
{
    BlockDims d = block_dims(mr);
    std::vector<float> taps(2 * d.n_os);
    CTBB_TRY(ctbb_load_filter(&mr, taps.data()));
    CTBB_TRY(prepare_ramp_filter(taps.data(), (int)d.n_os, &c.ramp, c.stream));
    StageScope scope(c, 2);
    return launch_ramp_filter(c.ramp, d_rebin, d.n_views * d.n_rows, c.stream);
}

// Where the rows of a block's views sit in the whole-scan paths' rows buffer:
// view j (= i + k n_half) is row off + j of the union's rows, except the
// views re-made from the block's own window (EdgePlan, dirty_view_runs),
// which sit at row patch + slot[j].
struct ViewRows {
    size_t off = 0;
    size_t patch = 0;
    std::vector<int> slot;  // per view: -1, or its row in the patch rows
    unsigned row(int j) const
    {
        if (j < (int)slot.size() && slot[(size_t)j] >= 0) return (unsigned)(patch + (size_t)slot[(size_t)j]);
        return (unsigned)(off + j);
    }
};

// The context's buffer for the backprojector's partial image sums, sized for
// a block of mr split into the most angle chunks a launch shape uses.
static int partial_scratch(Context &c, const struct recon_metadata &mr, void **ptr, size_t *bytes)
{
    const size_t need =
        (size_t)kMaxAngleChunks * mr.ri.n_slices_block * (size_t)mr.rp.nx * (size_t)mr.rp.ny * sizeof(float);
    CTBB_TRY(c.bp_partial.ensure(need));
    *ptr = c.bp_partial.ptr;
    *bytes = c.bp_partial.bytes;
    return CTBB_OK;
}

static int do_backproject(Context &c, const struct recon_metadata &mr, const float *d_rebin, float *d_block,
                          const ViewRows *rows = nullptr)
{
    BackprojectTables t;
    CTBB_TRY(build_backproject_tables(mr, &t));
    if (rows)
        for (int i = 0; i < t.n_half; ++i)
            for (int k = 0; k < t.nht; ++k) t.set_view_row(i, k, rows->row(i + k * t.n_half));
    CTBB_TRY(upload(c.bp_views, t.views, c.stream));
    CTBB_TRY(upload(c.bp_theta, t.theta, c.stream));
    CTBB_TRY(upload(c.bp_zpos, t.zpos, c.stream));
    void *part = nullptr;
    size_t part_bytes = 0;
    CTBB_TRY(partial_scratch(c, mr, &part, &part_bytes));
    StageScope scope(c, 3);
    return launch_backproject(mr, t, c.bp_views.as<float4>(), c.bp_theta.as<float>(), c.bp_zpos.as<float>(),
                              d_rebin, d_block, bp_zpt(), c.stream, nullptr, nullptr, part, part_bytes);
}

// The whole-scan paths' backprojection of one block from the context's rows:
// float32 rows (c.rebin) or footprint quads (c.quads, c.qscale).
static int backproject_scan_rows(Context &c, const struct recon_metadata &mr, float *d_block, const ViewRows &rows)
{
    if (c.storage == 0) return do_backproject(c, mr, c.rebin.as<float>(), d_block, &rows);
    BackprojectTables t;
    CTBB_TRY(build_backproject_tables(mr, &t));
    for (int i = 0; i < t.n_half; ++i)
        for (int k = 0; k < t.nht; ++k) t.set_view_row(i, k, rows.row(i + k * t.n_half));
    CTBB_TRY(upload(c.bp_views, t.views, c.stream));
    CTBB_TRY(upload(c.bp_theta, t.theta, c.stream));
    CTBB_TRY(upload(c.bp_zpos, t.zpos, c.stream));
    void *part = nullptr;
    size_t part_bytes = 0;
    CTBB_TRY(partial_scratch(c, mr, &part, &part_bytes));
    StageScope scope(c, 3);
    return launch_backproject(mr, t, c.bp_views.as<float4>(), c.bp_theta.as<float>(), c.bp_zpos.as<float>(),
                              reinterpret_cast<const float *>(c.quads.ptr), d_block, 8, c.stream,
                              c.qscale.as<float>(), nullptr, part, part_bytes);
}

// Ramp filter of rows [row0, row0 + n_lines) of the whole-scan rows buffer:
// float32 in place, or through the tensor cores into the footprint quads and
// scales at the same row index.
static int filter_scan_rows(Context &c, size_t row0, size_t n_lines, int rows_per_view, int n_os)
{
    StageScope scope(c, 2);
    if (c.storage == 0)
        return launch_ramp_filter(c.ramp, c.rebin.as<float>() + row0 * (size_t)n_os, n_lines, c.stream);
    return launch_ramp_tc(c.ramp_tc, c.rebin.as<float>() + row0 * (size_t)n_os, n_lines,
                          reinterpret_cast<__half *>(c.quads.ptr) + row0 * (size_t)n_os * 4,
                          c.qscale.as<float>() + row0, c.tc_work.ptr, c.stream, rows_per_view);
}

// Buffers and filter plan of the whole-scan paths for rows_total rows of the
// plan's geometry (the union's rows and the largest edge patch).
static int prepare_scan_rows(Context &c, const struct recon_metadata &mg, size_t rows_total, size_t union_lines)
{
    BlockDims d = block_dims(mg);
    std::vector<float> taps(2 * d.n_os);
    CTBB_TRY(ctbb_load_filter(&mg, taps.data()));
    CTBB_TRY(c.rebin.ensure(rows_total * d.n_os * sizeof(float)));
    if (c.storage == 0) return prepare_ramp_filter(taps.data(), (int)d.n_os, &c.ramp, c.stream);
    if (!ramp_tc_supported((int)d.n_os) || d.n_rows == 0 || 128 % d.n_rows != 0) {
        set_error("FP16 row storage needs rows of a multiple of 64 samples up to 1536 (here %zu) and detector rows "
                  "dividing 128 (here %zu)", d.n_os, d.n_rows);
        return CTBB_ERR_ARGUMENT;
    }
    CTBB_TRY(prepare_ramp_tc(taps.data(), (int)d.n_os, &c.ramp_tc, c.stream));
    CTBB_TRY(c.quads.ensure(rows_total * d.n_os * 4 * sizeof(__half)));
    CTBB_TRY(c.qscale.ensure(rows_total * sizeof(float)));
    return c.tc_work.ensure(ramp_tc_work_bytes(union_lines, (int)d.n_os));
}

static int do_finalize(Context &c, const struct recon_metadata &mr, const float *d_image, float *d_final, float mu_water)
{
    FinalizeTables t;
    CTBB_TRY(build_finalize_tables(mr, &t));
    CTBB_TRY(upload(c.fin_offsets, t.offsets, c.stream));
    CTBB_TRY(upload(c.fin_slices, t.slices, c.stream));
    CTBB_TRY(upload(c.fin_weights, t.weights, c.stream));
    StageScope scope(c, 4);
    return launch_finalize(mr, t, c.fin_offsets.as<int>(), c.fin_slices.as<int>(), c.fin_weights.as<float>(),
                           d_image, d_final, mu_water, c.stream);
}

}  // namespace ctbb

using namespace ctbb;

// --------------------------------------------------------------------------
// misc
// --------------------------------------------------------------------------

extern "C" const char *ctbb_version(void) { return "ctbangbang_gb300 0.1.0 (sm_103a)"; }

extern "C" int ctbb_set_stream(void *stream)
{
    Context &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    c.stream = reinterpret_cast<cudaStream_t>(stream);
    return CTBB_OK;
}

extern "C" uint64_t ctbb_kernel_launch_count(void) { return ctx().launches.load(); }

static int set_storage(Context &c, int mode)
{
    if (mode != CTBB_STORAGE_FP32 && mode != CTBB_STORAGE_FP16) {
        set_error("row storage %d is neither CTBB_STORAGE_FP32 nor CTBB_STORAGE_FP16", mode);
        return CTBB_ERR_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(c.mu);
    c.storage = mode;
    return CTBB_OK;
}

extern "C" int ctbb_set_storage(int mode)
{
    clear_error();
    return set_storage(ctx(), mode);
}

// Frees every work buffer, table, copy stream and staging buffer of c, on the
// device they live on.  device_sync: wait for the whole device first (the
// default context, whose stream the caller chooses); else for c's streams.
// unbind: forget the device, so that the next call may use another one.
static void release_context(Context &c, bool device_sync, bool unbind)
{
    int cur = 0, bound = c.device.load();
    cudaGetDevice(&cur);
    if (bound >= 0 && bound != cur) cudaSetDevice(bound);
    if (bound >= 0) {
        if (device_sync) {
            cudaDeviceSynchronize();
        } else {
            cudaStreamSynchronize(c.stream);
            if (c.copy_stream) cudaStreamSynchronize(c.copy_stream);
        }
    }
    for (DeviceBuffer *b : {&c.raw_in, &c.raw_in2, &c.raw_filt, &c.rebin, &c.block, &c.image, &c.final_stack,
                            &c.scratch, &c.bp_views, &c.bp_theta, &c.bp_zpos, &c.fin_offsets, &c.fin_slices,
                            &c.fin_weights, &c.edge_raw, &c.dirty, &c.bp_partial})
        b->release();
    if (c.rebin_tables.base) cudaFree(c.rebin_tables.base);
    c.rebin_tables = DeviceRebinTables{};
    if (c.ramp.d_spectrum) cudaFree(c.ramp.d_spectrum);
    c.ramp = RampFilterPlan{};
    release_ramp_tc(&c.ramp_tc);
    c.tc_work.release();
    c.quads.release();
    c.qscale.release();
    c.bp_tables.release();
    if (c.copy_stream) {
        for (int i = 0; i < 2; ++i) {
            cudaEventDestroy(c.copied[i]);
            cudaEventDestroy(c.consumed[i]);
            c.copied[i] = c.consumed[i] = nullptr;
        }
        for (cudaEvent_t e : c.chunk_copied) cudaEventDestroy(e);
        c.chunk_copied.clear();
        for (int i = 0; i < 2; ++i) {
            if (c.stage_free[i]) cudaEventDestroy(c.stage_free[i]);
            if (c.stage[i]) cudaFreeHost(c.stage[i]);
            c.stage_free[i] = nullptr;
            c.stage[i] = nullptr;
        }
        if (c.flags_ready) cudaEventDestroy(c.flags_ready);
        c.flags_ready = nullptr;
        c.stage_bytes = 0;
        if (c.flags_host) cudaFreeHost(c.flags_host);
        c.flags_host = nullptr;
        c.flags_host_bytes = 0;
        if (c.prep_stream) {
            cudaEventDestroy(c.prep_ready);
            cudaStreamDestroy(c.prep_stream);
            c.prep_stream = nullptr;
            c.prep_ready = nullptr;
        }
        cudaStreamDestroy(c.copy_stream);
        c.copy_stream = nullptr;
    }
    if (unbind) {
        c.sms = 0;
        c.device.store(-1);
    }
    if (bound >= 0 && bound != cur) cudaSetDevice(cur);
}

static void release_slots();

extern "C" int ctbb_release_workspace(void)
{
    Context &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    release_context(c, true, true);
    release_slots();
    return CTBB_OK;
}

// sizeof(struct recon_metadata) and member offsets, in the order the tests use.
extern "C" int ctbb_struct_layout(size_t *out, int n)
{
    size_t v[] = {
        sizeof(struct recon_metadata),
        offsetof(struct recon_metadata, flags), offsetof(struct recon_metadata, rp),
        offsetof(struct recon_metadata, ri), offsetof(struct recon_metadata, cg),
        offsetof(struct recon_metadata, ctd), offsetof(struct recon_metadata, tube_angles),
        offsetof(struct recon_metadata, table_positions), offsetof(struct recon_params, nx),
        offsetof(struct recon_params, table_dir), offsetof(struct recon_info, cb),
        offsetof(struct ct_geom, table_direction),
    };
    int m = (int)(sizeof(v) / sizeof(v[0]));
    for (int i = 0; i < n && i < m; ++i) out[i] = v[i];
    return m;
}

// --------------------------------------------------------------------------
// device-resident stages
// --------------------------------------------------------------------------

extern "C" int ctbb_adaptive_filter_device(const struct recon_metadata *mr, const float *d_in, float *d_out)
{
    clear_error();
    CTBB_TRY(check_mr(mr));
    Context &c = ctx();
    CTBB_TRY(require_device(c));
    std::lock_guard<std::mutex> lk(c.mu);
    return do_adaptive(c, *mr, d_in, d_out);
}

extern "C" int ctbb_rebin_device(const struct recon_metadata *mr, const float *d_raw, float *d_rebin)
{
    clear_error();
    CTBB_TRY(check_mr(mr));
    Context &c = ctx();
    CTBB_TRY(require_device(c));
    std::lock_guard<std::mutex> lk(c.mu);
    return do_rebin(c, *mr, d_raw, d_rebin);
}

extern "C" int ctbb_ramp_filter_device(float *d_lines, size_t n_lines, int n_os, const float *h_taps)
{
    clear_error();
    if (!d_lines || !h_taps || n_os <= 0) {
        set_error("ctbb_ramp_filter_device: bad argument");
        return CTBB_ERR_ARGUMENT;
    }
    CTBB_TRY(require_device(ctx()));
    Context &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    CTBB_TRY(prepare_ramp_filter(h_taps, n_os, &c.ramp, c.stream));
    return launch_ramp_filter(c.ramp, d_lines, n_lines, c.stream);
}

extern "C" int ctbb_ramp_filter_fp16_device(const float *d_lines, size_t n_lines, int n_os, const float *h_taps,
                                            int rows_per_view, void *d_out, float *d_scale)
{
    clear_error();
    if (!d_lines || !h_taps || !d_out || !d_scale || n_os <= 0) {
        set_error("ctbb_ramp_filter_fp16_device: bad argument");
        return CTBB_ERR_ARGUMENT;
    }
    if (!ramp_tc_supported(n_os)) {
        set_error("ctbb_ramp_filter_fp16_device: row length %d is not a multiple of 64 up to 1536", n_os);
        return CTBB_ERR_ARGUMENT;
    }
    if (rows_per_view < 0 || (rows_per_view > 0 && 128 % rows_per_view != 0)) {
        set_error("ctbb_ramp_filter_fp16_device: rows per view %d must divide 128", rows_per_view);
        return CTBB_ERR_ARGUMENT;
    }
    Context &c = ctx();
    CTBB_TRY(require_device(c));
    std::lock_guard<std::mutex> lk(c.mu);
    CTBB_TRY(prepare_ramp_tc(h_taps, n_os, &c.ramp_tc, c.stream));
    CTBB_TRY(c.tc_work.ensure(ramp_tc_work_bytes(n_lines, n_os)));
    StageScope scope(c, 2);
    CTBB_TRY(launch_ramp_tc(c.ramp_tc, d_lines, n_lines, static_cast<__half *>(d_out), d_scale, c.tc_work.ptr,
                            c.stream, rows_per_view));
    return ramp_tc_check(c.ramp_tc, c.stream);
}

extern "C" int ctbb_backproject_fp16_device(const struct recon_metadata *mr, const void *d_quads,
                                            const float *d_scale, float *d_block)
{
    clear_error();
    CTBB_TRY(check_mr(mr));
    if (!d_quads || !d_scale || !d_block) {
        set_error("ctbb_backproject_fp16_device: null buffer");
        return CTBB_ERR_ARGUMENT;
    }
    Context &c = ctx();
    CTBB_TRY(require_device(c));
    std::lock_guard<std::mutex> lk(c.mu);
    BackprojectTables t;
    CTBB_TRY(build_backproject_tables(*mr, &t));
    CTBB_TRY(upload(c.bp_views, t.views, c.stream));
    CTBB_TRY(upload(c.bp_theta, t.theta, c.stream));
    CTBB_TRY(upload(c.bp_zpos, t.zpos, c.stream));
    void *part = nullptr;
    size_t part_bytes = 0;
    CTBB_TRY(partial_scratch(c, *mr, &part, &part_bytes));
    StageScope scope(c, 3);
    return launch_backproject(*mr, t, c.bp_views.as<float4>(), c.bp_theta.as<float>(), c.bp_zpos.as<float>(),
                              static_cast<const float *>(d_quads), d_block, 8, c.stream, d_scale, nullptr, part,
                              part_bytes);
}

extern "C" int ctbb_backproject_device(const struct recon_metadata *mr, const float *d_rebin, float *d_block)
{
    clear_error();
    CTBB_TRY(check_mr(mr));
    Context &c = ctx();
    CTBB_TRY(require_device(c));
    std::lock_guard<std::mutex> lk(c.mu);
    return do_backproject(c, *mr, d_rebin, d_block);
}

extern "C" int ctbb_finalize_device(const struct recon_metadata *mr, const float *d_image, float *d_final,
                                    float mu_water)
{
    clear_error();
    CTBB_TRY(check_mr(mr));
    Context &c = ctx();
    CTBB_TRY(require_device(c));
    std::lock_guard<std::mutex> lk(c.mu);
    return do_finalize(c, *mr, d_image, d_final, mu_water);
}

extern "C" size_t ctbb_workspace_bytes(const struct recon_metadata *mr)
{
    if (check_mr(mr)) return 0;
    BlockDims d = block_dims(*mr);
    // raw window (copy) + filtered raw + rebin + image stack + the
    // backprojector's angle-chunk partial sums of a block; pull windows of
    // later blocks can be up to 128 frames longer than the planned first one.
    size_t frame = d.n_rows_raw * d.n_channels;
    size_t raw = (d.n_proj_pull + 256) * frame * sizeof(float);
    size_t rebin = ((d.n_proj_pull + 256) / d.n_ffs) * d.n_rows * d.n_os * sizeof(float);
    size_t image = (size_t)mr->rp.nx * mr->rp.ny * mr->ri.n_slices_recon * sizeof(float);
    size_t partial = (size_t)kMaxAngleChunks * mr->rp.nx * mr->rp.ny * mr->ri.n_slices_block * sizeof(float);
    return 2 * raw + rebin + image + partial;
}

// Runs a reconstruction body and then waits for the context's copy and
// compute streams, so that once a call has returned -- also one that failed
// halfway, say on a missing filter file after its first copies were enqueued
// -- no copy from the caller's host buffer and no kernel writing the caller's
// output is still in flight.  After a successful body both are idle already;
// a device fault that only surfaces in this wait is the call's error (a
// failing body keeps its own first error).
template <class Body>
static int drained(Context &c, Body &&body)
{
    int st = body();
    cudaError_t e1 = c.copy_stream ? cudaStreamSynchronize(c.copy_stream) : cudaSuccess;
    const cudaError_t e0 = c.prep_stream ? cudaStreamSynchronize(c.prep_stream) : cudaSuccess;
    if (e1 == cudaSuccess) e1 = e0;
    cudaError_t e2 = cudaStreamSynchronize(c.stream);
    if (st == CTBB_OK && (e1 != cudaSuccess || e2 != cudaSuccess)) {
        set_error("device work of this call failed: %s",
                  cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
        return CTBB_ERR_CUDA;
    }
    return st;
}

static int reconstruct_device_in(Context &c, struct recon_metadata *mr, const float *d_scan, float *d_final,
                                       float mu_water)
{
    clear_error();
    if (!mr || !d_scan || !d_final || !mr->table_positions) {
        set_error("ctbb_reconstruct_device: metadata not configured or null buffer");
        return CTBB_ERR_ARGUMENT;
    }
    CTBB_TRY(check_mr(mr));
    CTBB_TRY(require_device(c));
    std::lock_guard<std::mutex> lk(c.mu);
    return drained(c, [&]() -> int {
        const size_t frame = mr->cg.n_rows_raw * mr->cg.n_channels;
        const size_t n_readings = (size_t)mr->rp.n_readings;
        const size_t plane = (size_t)mr->rp.nx * mr->rp.ny;
        const size_t n_block = mr->ri.n_slices_block;
        CTBB_TRY(c.image.ensure(plane * mr->ri.n_slices_recon * sizeof(float)));
        mr->ri.cb.block_idx = 0;
        for (size_t b = 0; b < mr->ri.n_blocks; ++b) {
            struct recon_info ri;
            CTBB_TRY(plan_next_block(*mr, &ri));
            mr->ri = ri;
            BlockDims d = block_dims(*mr);
            // the block's pull window: a view into the resident scan when it lies
            // inside the data, else a zero-filled copy (frames past either end read 0)
            long long s0 = (long long)(int)mr->ri.idx_pull_start;
            long long s1 = s0 + (long long)d.n_proj_pull;
            const float *d_win = nullptr;
            if (s0 >= 0 && s1 <= (long long)n_readings) {
                d_win = d_scan + (size_t)s0 * frame;
            } else {
                CTBB_TRY(c.raw_in.ensure(d.raw_elems() * sizeof(float)));
                CTBB_CUDA_TRY(cudaMemsetAsync(c.raw_in.ptr, 0, d.raw_elems() * sizeof(float), c.stream));
                long long a = s0 < 0 ? 0 : s0, e = s1 > (long long)n_readings ? (long long)n_readings : s1;
                if (e > a)
                    CTBB_CUDA_TRY(cudaMemcpyAsync(c.raw_in.as<float>() + (size_t)(a - s0) * frame,
                                                  d_scan + (size_t)a * frame, (size_t)(e - a) * frame * sizeof(float),
                                                  cudaMemcpyDeviceToDevice, c.stream));
                d_win = c.raw_in.as<float>();
            }
            CTBB_TRY(c.raw_filt.ensure(d.raw_elems() * sizeof(float)));
            CTBB_TRY(do_adaptive(c, *mr, d_win, c.raw_filt.as<float>()));
            CTBB_TRY(c.rebin.ensure(d.rebin_elems() * sizeof(float)));
            CTBB_TRY(do_rebin(c, *mr, c.raw_filt.as<float>(), c.rebin.as<float>()));
            CTBB_TRY(do_filter(c, *mr, c.rebin.as<float>()));
            float *slab = c.image.as<float>() + b * n_block * plane;
            CTBB_TRY(do_backproject(c, *mr, c.rebin.as<float>(), slab));
        }
        CTBB_TRY(do_finalize(c, *mr, c.image.as<float>(), d_final, mu_water));
        CTBB_CUDA_TRY(cudaStreamSynchronize(c.stream));
        return CTBB_OK;
    });
}

extern "C" int ctbb_reconstruct_device(struct recon_metadata *mr, const float *d_scan, float *d_final,
                                       float mu_water)
{
    return reconstruct_device_in(ctx(), mr, d_scan, d_final, mu_water);
}

// Every block's plan, as the block loop makes them, and the union of their
// pull windows [g0, g1) as one plan mg (the whole-scan paths).
static int plan_union(struct recon_metadata *mr, std::vector<struct recon_info> *blocks, long long *g0_out,
                      long long *g1_out, struct recon_metadata *mg)
{
    blocks->assign(mr->ri.n_blocks, recon_info{});
    mr->ri.cb.block_idx = 0;
    long long g0 = 0, g1 = 0;
    for (size_t b = 0; b < blocks->size(); ++b) {
        CTBB_TRY(plan_next_block(*mr, &(*blocks)[b]));
        mr->ri = (*blocks)[b];
        long long s0 = (long long)(int)(*blocks)[b].idx_pull_start;
        long long s1 = s0 + (long long)(*blocks)[b].n_proj_pull;
        g0 = b == 0 ? s0 : std::min(g0, s0);
        g1 = b == 0 ? s1 : std::max(g1, s1);
    }
    if (blocks->empty()) {
        set_error("whole scan: the plan has no blocks");
        return CTBB_ERR_STATE;
    }
    const long long n_ffs = (long long)(*blocks)[0].n_ffs;
    for (const auto &ri : *blocks)
        if (((long long)(int)ri.idx_pull_start - g0) % n_ffs != 0) {
            set_error("whole scan: pull windows not aligned to the focal-spot cycle");
            return CTBB_ERR_STATE;
        }
    *mg = *mr;
    mg->ri = (*blocks)[0];
    mg->ri.idx_pull_start = (size_t)g0;
    mg->ri.n_proj_pull = (size_t)(g1 - g0);
    *g0_out = g0;
    *g1_out = g1;
    return CTBB_OK;
}

// first rebinned view of block b in the union's rebinned rows
static size_t union_view_offset(const struct recon_info &ri, long long g0)
{
    return (size_t)(((long long)(int)ri.idx_pull_start - g0) / (long long)ri.n_ffs);
}

// Views of one block that the whole-scan paths re-make from the block's own
// pull window.  The reference filters every block's window on its own
// (src/main.cu:222, the window of src/setup.cu:637-661), and the adaptive
// filter's 18- and 180-degree statistics (include/preprocessing.cuh:87-206)
// stop at that window's ends.  Within adaptive_filter_edge_reach frames of a
// window end that is not also an end of the union window, the block's
// filtered frames can therefore differ from the union's; elsewhere they are
// the same.  The block's views [0, d0) and [d1, n_used) read such frames
// (rebin_frames_needed bounds a view's frames from above; a view j reads no
// frame below n_ffs (j - 2)); they are rebinned from frames [0, fa) and
// [fb, P) of the block's window filtered with the block's own thresholds.
struct EdgePlan {
    int d0 = 0, d1 = 0, n_used = 0, fa = 0, fb = 0;
    bool any() const { return d0 > 0 || d1 < n_used; }
    int n_patch() const { return d0 + (n_used - d1); }
};

static EdgePlan edge_plan(const struct recon_metadata &mb, long long g0, long long g1)
{
    EdgePlan e;
    BlockDims d = block_dims(mb);
    const long long P = (long long)d.n_proj_pull, n_ffs = (long long)d.n_ffs;
    const long long add = (long long)mb.cg.add_projections;
    const long long s = (long long)(int)mb.ri.idx_pull_start;
    const long long reach = adaptive_filter_edge_reach(mb);
    e.n_used = d.n_half_turns * (int)(mb.cg.n_proj_turn / 2);
    e.d1 = e.n_used;
    if (s > g0) e.d0 = (int)std::min<long long>(e.n_used, (reach + n_ffs - 1) / n_ffs + 2);
    if (s + P < g1) {
        long long last_clean = (P - reach) >= 0 ? (P - reach) / n_ffs - 2 * add - 2 : -1;
        e.d1 = (int)std::max<long long>(e.d0, std::min<long long>(e.n_used, last_clean + 1));
    }
    e.fa = e.d0 > 0 ? (int)std::min(P, n_ffs * (e.d0 - 1 + 2 * add + 2)) : 0;
    e.fb = e.d1 < e.n_used ? (int)std::max(0LL, n_ffs * (e.d1 - 2)) : (int)P;
    if (e.fb < e.fa) e.fb = e.fa;
    return e;
}

// Largest pull window and edge patch (views) over the blocks of a plan; the
// sums of the edge patches and of the pull windows of blocks with edge views.
static void edge_extent(const struct recon_metadata &mr, const std::vector<struct recon_info> &blocks,
                        long long g0, long long g1, size_t *max_pull, size_t *max_patch, size_t *sum_patch = nullptr,
                        size_t *sum_edge_pull = nullptr)
{
    *max_pull = 0;
    *max_patch = 0;
    if (sum_patch) *sum_patch = 0;
    if (sum_edge_pull) *sum_edge_pull = 0;
    for (const auto &ri : blocks) {
        struct recon_metadata mb = mr;
        mb.ri = ri;
        EdgePlan e = edge_plan(mb, g0, g1);
        *max_pull = std::max(*max_pull, (size_t)ri.n_proj_pull);
        *max_patch = std::max(*max_patch, (size_t)e.n_patch());
        if (sum_patch) *sum_patch += (size_t)e.n_patch();
        if (sum_edge_pull && e.any()) *sum_edge_pull += (size_t)ri.n_proj_pull;
    }
}

// First step of a block's edge views: its window's thresholds from its own
// statistics (the frames' maxima are the union's, d_union_sup at the block's
// offset; d_block_scratch holds 6 P floats), and per frame of the window
// whether its filtered value can differ from the union's (d_dirty, P bytes),
// given the union's thresholds d_union_thr.
static int edge_dirty_frames(Context &c, const struct recon_metadata &mb, const EdgePlan &e,
                             const float *d_union_raw, const float *d_union_sup, const float *d_union_thr,
                             long long g0, long long g1, float *d_block_scratch, unsigned char *d_dirty)
{
    BlockDims d = block_dims(mb);
    const size_t frame = d.n_rows_raw * d.n_channels;
    const long long sb = (long long)(int)mb.ri.idx_pull_start - g0;
    const int lo_edge = sb > 0 ? 1 : 0;
    const int hi_edge = (long long)(int)mb.ri.idx_pull_start + (long long)d.n_proj_pull < g1 ? 1 : 0;
    StageScope scope(c, 0);
    CTBB_TRY(launch_adaptive_filter_ends_thresholds(mb, d_union_raw + (size_t)sb * frame, d_union_sup + sb,
                                                    d_block_scratch, e.fa, e.fb, c.stream));
    return launch_adaptive_filter_dirty(mb, d_union_sup + sb, d_union_thr + sb, d_block_scratch, e.fa, e.fb,
                                        lo_edge, hi_edge, d_dirty, c.stream);
}

// The block's rebin tables: the union's with the block's own window length
// and float view-axis coordinates, as its block loop.
static RebinTables block_rebin_tables(const RebinTables &rt, const BlockDims &d)
{
    RebinTables tb = rt;
    tb.split_view_coord = 0;
    tb.n_proj = (int)(d.n_proj_pull / d.n_ffs);
    tb.n_views = tb.n_proj - 2 * tb.add_projections;
    return tb;
}

// Runs [j0, j1) of the block's edge views that read a frame whose filtered
// value can differ from the union's (dirty, one byte per frame of the
// block's window): view j reads frames [n_ffs (j - 2), rebin_frames_needed(j)).
// Runs closer than kRunGap views are joined (fewer launches; a joined view
// re-made from the block's window is as exact as the union's).
static std::vector<std::pair<int, int>> dirty_view_runs(const EdgePlan &e, const RebinTables &tb,
                                                        const unsigned char *dirty, int P)
{
    constexpr int kRunGap = 32;
    std::vector<int> cum((size_t)P + 1, 0);
    for (int f = 0; f < P; ++f) cum[(size_t)f + 1] = cum[(size_t)f] + (dirty[f] ? 1 : 0);
    std::vector<std::pair<int, int>> runs;
    if (cum[(size_t)P] == 0) return runs;
    auto scan = [&](int v0, int v1) {
        int run0 = -1, last = -1;
        for (int j = v0; j < v1; ++j) {
            const int a = std::max(0, tb.n_ffs * (j - 2));
            const int b = std::min(P, rebin_frames_needed(tb, j));
            if (b <= a || cum[(size_t)b] == cum[(size_t)a]) continue;
            if (run0 >= 0 && j - last <= kRunGap) {
                last = j;
                continue;
            }
            if (run0 >= 0) runs.emplace_back(run0, last + 1);
            run0 = last = j;
        }
        if (run0 >= 0) runs.emplace_back(run0, last + 1);
    };
    scan(0, e.d0);
    scan(e.d1, e.n_used);
    return runs;
}

// Re-makes the runs of block mb's edge views: their frames of the block's
// window filtered with the block's own thresholds (left in d_block_scratch
// by edge_dirty_frames) into c.edge_raw, the views rebinned from there into
// the rows from patch_view on, in run order, and ramp-filtered; vr->slot
// records where each landed and *n_made counts the views.
static int run_edge_patch(Context &c, const struct recon_metadata &mb, const RebinTables &rt,
                          const std::vector<std::pair<int, int>> &runs, const float *d_union_raw,
                          const float *d_union_sup, long long g0, float *d_block_scratch, size_t patch_view,
                          ViewRows *vr, size_t *n_made)
{
    *n_made = 0;
    if (runs.empty()) return CTBB_OK;
    BlockDims d = block_dims(mb);
    const size_t frame = d.n_rows_raw * d.n_channels;
    const size_t view_elems = d.n_rows * d.n_os;
    const long long sb = (long long)(int)mb.ri.idx_pull_start - g0;
    const int P = (int)d.n_proj_pull;
    const RebinTables tb = block_rebin_tables(rt, d);
    size_t slot = 0;
    for (const auto &r : runs) {
        const int f0 = std::max(0, tb.n_ffs * (r.first - 2));
        const int f1 = std::min(P, rebin_frames_needed(tb, r.second - 1));
        {
            StageScope scope(c, 0);
            CTBB_TRY(launch_adaptive_filter_output(mb, d_union_raw + (size_t)sb * frame, c.edge_raw.as<float>(),
                                                   d_union_sup + sb, d_block_scratch, f0, f1, c.stream));
        }
        // view v of the run lands in row patch_view + slot + (v - r.first)
        float *d_out = c.rebin.as<float>() + (patch_view + slot) * view_elems - (size_t)r.first * view_elems;
        {
            StageScope scope(c, 1);
            CTBB_TRY(launch_rebin(tb, c.rebin_tables, c.edge_raw.as<float>(), d_out, c.stream, r.first, r.second));
        }
        const size_t n = (size_t)(r.second - r.first);
        CTBB_TRY(filter_scan_rows(c, (patch_view + slot) * d.n_rows, n * d.n_rows, (int)d.n_rows, (int)d.n_os));
        for (int j = r.first; j < r.second; ++j) vr->slot[(size_t)j] = (int)(slot + (size_t)(j - r.first));
        slot += n;
    }
    *n_made = slot;
    return CTBB_OK;
}

// Device bytes the whole-scan paths (scan_device / scan_host / scan_file)
// hold for this plan: the union window raw and filtered, its rebinned rows,
// the adaptive filter's statistics, the image and final stacks, the
// backprojector's angle-chunk partial sums of a block, plus 8 MiB for tables
// and staging slack.  0 if the plan is not usable.
extern "C" size_t ctbb_scan_workspace_bytes(const struct recon_metadata *mr)
{
    if (!mr || check_mr(mr) || !mr->table_positions) return 0;
    struct recon_metadata m = *mr;  // plan_union advances the block index
    std::vector<struct recon_info> blocks;
    long long g0 = 0, g1 = 0;
    struct recon_metadata mg;
    if (plan_union(&m, &blocks, &g0, &g1, &mg) != CTBB_OK) return 0;
    BlockDims dg = block_dims(mg);
    const size_t plane = (size_t)mr->rp.nx * mr->rp.ny;
    const int n_final = ctbb_n_slices_final(mr);
    size_t max_pull = 0, max_patch = 0, sum_patch = 0, sum_edge_pull = 0;
    edge_extent(m, blocks, g0, g1, &max_pull, &max_patch, &sum_patch, &sum_edge_pull);
    const size_t frame = dg.n_rows_raw * dg.n_channels, view_elems = dg.n_rows * dg.n_os;
    return (2 * dg.raw_elems() + dg.rebin_elems() + sum_patch * view_elems + max_pull * frame +
            adaptive_filter_scratch_floats(dg.n_proj_pull) +
            adaptive_filter_scratch_floats(std::max(max_pull, sum_edge_pull)) + plane * mr->ri.n_slices_recon +
            plane * (size_t)(n_final > 0 ? n_final : 1) +
            (size_t)kMaxAngleChunks * mr->ri.n_slices_block * plane) * sizeof(float) +
           sum_edge_pull + ((size_t)8 << 20);
}


// Whole scan with one resident rebinned scan: the union of all blocks' pull
// windows is adaptive-filtered, rebinned and ramp-filtered once, and every
// block backprojects from its own offset into that rebinned scan (consecutive
// windows overlap by most of their frames, which the block loop processes
// again for every block).  Differs from the block loop only in the adaptive
// filter's 18- and 180-degree statistics windows, which here are not cut at
// the edges of each block's window.
// A whole scan prepared for its backprojections (prepare_scan_device): the
// blocks' plans, where each block's views sit in the context's rows, and the
// offsets of each block's tables (views, theta, slice positions) in
// c.bp_tables.
struct ScanPrep {
    std::vector<struct recon_info> blocks;
    std::vector<ViewRows> rows;
    std::vector<BackprojectTables> tables;
    std::vector<size_t> table_off;  // floats: views (16-byte aligned), then theta, then zpos
};

// Union window adaptive-filtered, rebinned and ramp-filtered once, every
// block's edge views re-made into rows of their own after the union's, and
// every block's tables uploaded, on c's buffers and stream.  The caller holds
// c.mu.  mr->ri is left at the last block.
static int prepare_scan_device(Context &c, struct recon_metadata *mr, const float *d_scan, ScanPrep *prep)
{
    const size_t frame = mr->cg.n_rows_raw * mr->cg.n_channels;
    const long long n_readings = (long long)mr->rp.n_readings;
    const size_t plane = (size_t)mr->rp.nx * mr->rp.ny;
    long long g0 = 0, g1 = 0;
    struct recon_metadata mg;
    CTBB_TRY(plan_union(mr, &prep->blocks, &g0, &g1, &mg));
    const std::vector<struct recon_info> &blocks = prep->blocks;
    BlockDims dg = block_dims(mg);
    const float *d_win = nullptr;
    if (g0 >= 0 && g1 <= n_readings) {
        d_win = d_scan + (size_t)g0 * frame;
    } else {
        CTBB_TRY(c.raw_in.ensure(dg.raw_elems() * sizeof(float)));
        CTBB_CUDA_TRY(cudaMemsetAsync(c.raw_in.ptr, 0, dg.raw_elems() * sizeof(float), c.stream));
        long long a = g0 < 0 ? 0 : g0, e = g1 > n_readings ? n_readings : g1;
        if (e > a)
            CTBB_CUDA_TRY(cudaMemcpyAsync(c.raw_in.as<float>() + (size_t)(a - g0) * frame, d_scan + (size_t)a * frame,
                                          (size_t)(e - a) * frame * sizeof(float), cudaMemcpyDeviceToDevice,
                                          c.stream));
        d_win = c.raw_in.as<float>();
    }
    CTBB_TRY(c.image.ensure(plane * mr->ri.n_slices_recon * sizeof(float)));
    CTBB_TRY(c.raw_filt.ensure(dg.raw_elems() * sizeof(float)));
    size_t max_pull = 0, max_patch = 0, sum_patch = 0;
    edge_extent(*mr, blocks, g0, g1, &max_pull, &max_patch, &sum_patch);
    // scratch: the union's statistics, then each block's (6 P floats each);
    // dirty: one byte per frame of each block's window
    const size_t af_union = adaptive_filter_scratch_floats(dg.n_proj_pull);
    std::vector<EdgePlan> plans(blocks.size());
    std::vector<size_t> af_off(blocks.size(), 0), dirty_off(blocks.size(), 0);
    size_t af_total = af_union, dirty_total = 0;
    for (size_t b = 0; b < blocks.size(); ++b) {
        mr->ri = blocks[b];
        plans[b] = edge_plan(*mr, g0, g1);
        if (!plans[b].any()) continue;
        af_off[b] = af_total;
        dirty_off[b] = dirty_total;
        af_total += adaptive_filter_scratch_floats(blocks[b].n_proj_pull);
        dirty_total += blocks[b].n_proj_pull;
    }
    CTBB_TRY(c.scratch.ensure(af_total * sizeof(float)));
    if (dirty_total) CTBB_TRY(c.dirty.ensure(dirty_total));
    float *d_union_sup = c.scratch.as<float>();
    const float *d_union_thr = c.scratch.as<float>() + 5 * (size_t)dg.n_proj_pull;  // af_params' thr slot
    {
        StageScope scope(c, 0);
        CTBB_TRY(launch_adaptive_filter(mg, d_win, c.raw_filt.as<float>(), c.scratch.as<float>(), c.stream));
    }
    CTBB_TRY(prepare_scan_rows(c, mg, (dg.n_views + sum_patch) * dg.n_rows, dg.n_views * dg.n_rows));
    RebinTables rt;
    CTBB_TRY(build_rebin_tables(mg, &rt));
    rt.split_view_coord = 1;  // the union's frame offsets are large
    CTBB_TRY(upload_rebin_tables(rt, &c.rebin_tables, c.stream));
    {
        StageScope scope(c, 1);
        CTBB_TRY(launch_rebin(rt, c.rebin_tables, c.raw_filt.as<float>(), c.rebin.as<float>(), c.stream));
    }
    // each block's edge frames that can filter differently from the union
    for (size_t b = 0; b < blocks.size(); ++b) {
        if (!plans[b].any()) continue;
        mr->ri = blocks[b];
        CTBB_TRY(edge_dirty_frames(c, *mr, plans[b], d_win, d_union_sup, d_union_thr, g0, g1,
                                   c.scratch.as<float>() + af_off[b], c.dirty.as<unsigned char>() + dirty_off[b]));
    }
    CTBB_TRY(filter_scan_rows(c, 0, dg.n_views * dg.n_rows, (int)dg.n_rows, (int)dg.n_os));
    // the flags come back once the union is filtered (the copy waits for the
    // stream; the device has the union's rows to make meanwhile)
    std::vector<unsigned char> dirty(dirty_total);
    if (dirty_total) {
        CTBB_CUDA_TRY(cudaMemcpyAsync(dirty.data(), c.dirty.ptr, dirty_total, cudaMemcpyDeviceToHost, c.stream));
        CTBB_CUDA_TRY(cudaStreamSynchronize(c.stream));
    }
    if (max_patch) CTBB_TRY(c.edge_raw.ensure(max_pull * dg.n_rows_raw * dg.n_channels * sizeof(float)));
    // the re-made edge views of every block in rows of their own, and its tables
    prep->rows.assign(blocks.size(), ViewRows{});
    prep->tables.assign(blocks.size(), BackprojectTables{});
    prep->table_off.assign(blocks.size(), 0);
    std::vector<float> host_tables;
    size_t patch_view = dg.n_views;
    for (size_t b = 0; b < blocks.size(); ++b) {
        mr->ri = blocks[b];
        ViewRows &vr = prep->rows[b];
        vr.off = union_view_offset(blocks[b], g0);
        vr.patch = patch_view;
        const EdgePlan &e = plans[b];
        if (e.any()) {
            BlockDims db = block_dims(*mr);
            const auto runs = dirty_view_runs(e, block_rebin_tables(rt, db), dirty.data() + dirty_off[b],
                                              (int)db.n_proj_pull);
            vr.slot.assign((size_t)e.n_used, -1);
            size_t made = 0;
            CTBB_TRY(run_edge_patch(c, *mr, rt, runs, d_win, d_union_sup, g0, c.scratch.as<float>() + af_off[b],
                                    patch_view, &vr, &made));
            patch_view += made;
        }
        BackprojectTables &t = prep->tables[b];
        CTBB_TRY(build_backproject_tables(*mr, &t));
        for (int i = 0; i < t.n_half; ++i)
            for (int k = 0; k < t.nht; ++k) t.set_view_row(i, k, vr.row(i + k * t.n_half));
        size_t off = (host_tables.size() + 3) & ~(size_t)3;
        prep->table_off[b] = off;
        host_tables.resize(off);
        host_tables.insert(host_tables.end(), t.views.begin(), t.views.end());
        host_tables.insert(host_tables.end(), t.theta.begin(), t.theta.end());
        host_tables.insert(host_tables.end(), t.zpos.begin(), t.zpos.end());
    }
    return upload(c.bp_tables, host_tables, c.stream);
}

// Kernel parameters of block b of a prepared scan (its image slab d_block).
static int prepared_block_params(Context &c, const struct recon_metadata &mb, const ScanPrep &prep, size_t b,
                                 float *d_block, const BpShape &shape, BpParams *p)
{
    const BackprojectTables &t = prep.tables[b];
    const float *base = c.bp_tables.as<float>() + prep.table_off[b];
    const float4 *d_views = reinterpret_cast<const float4 *>(base);
    const float *d_theta = base + t.views.size();
    const float *d_zpos = d_theta + t.theta.size();
    const float *rows = c.storage ? reinterpret_cast<const float *>(c.quads.ptr) : c.rebin.as<float>();
    const float *vscale = c.storage ? c.qscale.as<float>() : nullptr;
    return make_backproject_params(mb, t, d_views, d_theta, d_zpos, rows, d_block, vscale, shape, p);
}

// ---- autotuner -------------------------------------------------------------
// Picks a backprojector launch shape (slices per thread, CTA size, CTAs per
// SM, CTA width) for each geometry class -- image size, slices per block, row
// length, detector rows, half turns, row storage -- by timing every candidate
// once on the first block of that class (CUDA events on the context's
// stream; the block is recomputed by the chosen shape afterwards), and caches
// the choice for the process.

struct TuneKey {
    int nx, ny, n_slices, nos, n_rows, nht, quad;
    bool operator<(const TuneKey &o) const
    {
        return std::tie(nx, ny, n_slices, nos, n_rows, nht, quad) <
               std::tie(o.nx, o.ny, o.n_slices, o.nos, o.n_rows, o.nht, o.quad);
    }
};

struct TuneEntry {
    BpShape shape;
    double ms[8] = {0};  // candidate times, in backproject_shape_candidates order
    int n = 0;
};

static std::mutex g_tune_mu;
static std::map<TuneKey, TuneEntry> g_tuned;

// Timed launches per candidate (the fastest counts): CTBB_TUNE_REPS, 1 to 9.
static int tune_reps()
{
    static int v = [] {
        const char *e = getenv("CTBB_TUNE_REPS");
        const int r = e ? atoi(e) : 1;
        return r < 1 ? 1 : (r > 9 ? 9 : r);
    }();
    return v;
}

static int tuned_shape(Context &c, const BpParams &p_any, const BpShape &fallback, BpShape *out)
{
    const bool quad = p_any.vscale != nullptr;
    const TuneKey key{p_any.nx, p_any.ny, p_any.n_slices, p_any.nos, p_any.n_rows, p_any.nht, quad ? 1 : 0};
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            *out = it->second.shape;
            return CTBB_OK;
        }
    }
    std::vector<BpShape> cand = backproject_shape_candidates(quad);
    TuneEntry best;
    best.shape = fallback;
    double best_ms = 1e30;
    cudaEvent_t e0 = pooled_event(c), e1 = pooled_event(c);
    for (size_t k = 0; k < cand.size() && k < 8; ++k) {
        if (cand[k].col && p_any.nht > kColumnMaxHalfTurns) continue;  // the window does not fit
        BpParams p = p_any;
        p.col_zpt = cand[k].col ? cand[k].zpt : 0;
        p.warp_w = cand[k].warp_w;
        p.cta_w = std::max(cand[k].cta_w, p.warp_w);
        if (cand[k].threads / p.cta_w < 32 / p.warp_w) p.cta_w = (cand[k].threads / 32) * p.warp_w;
        const size_t part = backproject_partial_bytes(p, cand[k]);
        if (part) CTBB_TRY(c.bp_partial.ensure(part));
        auto launch = [&]() {
            return launch_backproject_params(p, cand[k], c.stream, c.bp_partial.ptr, c.bp_partial.bytes);
        };
        CTBB_TRY(launch());  // warm-up (module load, caches)
        float ms = 1e30f;
        for (int r = 0; r < tune_reps(); ++r) {
            CTBB_CUDA_TRY(cudaEventRecord(e0, c.stream));
            CTBB_TRY(launch());
            CTBB_CUDA_TRY(cudaEventRecord(e1, c.stream));
            CTBB_CUDA_TRY(cudaEventSynchronize(e1));
            float t = 0.0f;
            CTBB_CUDA_TRY(cudaEventElapsedTime(&t, e0, e1));
            ms = std::min(ms, t);
        }
        best.ms[k] = ms;
        best.n = (int)k + 1;
        if (ms < best_ms) {
            best_ms = ms;
            best.shape = cand[k];
        }
    }
    c.event_pool.push_back(e0);
    c.event_pool.push_back(e1);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[key] = best;
    *out = best.shape;
    return CTBB_OK;
}

static int reconstruct_scan_device_in(Context &c, struct recon_metadata *mr, const float *d_scan, float *d_final,
                                            float mu_water)
{
    clear_error();
    if (!mr || !d_scan || !d_final || !mr->table_positions) {
        set_error("ctbb_reconstruct_scan_device: metadata not configured or null buffer");
        return CTBB_ERR_ARGUMENT;
    }
    CTBB_TRY(check_mr(mr));
    CTBB_TRY(require_device(c));
    std::lock_guard<std::mutex> lk(c.mu);
    return drained(c, [&]() -> int {
        const size_t plane = (size_t)mr->rp.nx * mr->rp.ny;
        const size_t n_block = mr->ri.n_slices_block;
        ScanPrep prep;
        CTBB_TRY(prepare_scan_device(c, mr, d_scan, &prep));
        for (size_t b = 0; b < prep.blocks.size(); ++b) {
            mr->ri = prep.blocks[b];
            float *slab = c.image.as<float>() + b * n_block * plane;
            const BpShape fallback = window_bp_shape(bp_zpt(), c.storage != 0, prep.tables[b].nht);
            BpParams p;
            CTBB_TRY(prepared_block_params(c, *mr, prep, b, slab, fallback, &p));
            BpShape shape = fallback;
            if (c.autotune) {
                CTBB_TRY(tuned_shape(c, p, fallback, &shape));
                CTBB_TRY(prepared_block_params(c, *mr, prep, b, slab, shape, &p));
            }
            const size_t part = backproject_partial_bytes(p, shape);
            if (part) CTBB_TRY(c.bp_partial.ensure(part));
            StageScope scope(c, 3);
            CTBB_TRY(launch_backproject_params(p, shape, c.stream, c.bp_partial.ptr, c.bp_partial.bytes));
        }
        CTBB_TRY(do_finalize(c, *mr, c.image.as<float>(), d_final, mu_water));
        CTBB_CUDA_TRY(cudaStreamSynchronize(c.stream));
        if (c.storage) CTBB_TRY(ramp_tc_check(c.ramp_tc, c.stream));
        return CTBB_OK;
    });
}

// ---- many whole scans, one backprojection launch ---------------------------
// Every scan of a batch is prepared (union filtered, rebinned, ramp-filtered,
// edge views re-made, tables uploaded) into a slot of its own -- rows, tables,
// image -- and then the blocks of all scans are backprojected together: one
// launch per launch shape (the autotuner's choice for each geometry class),
// whose CTAs run over the tiles of every block in turn, so the small blocks of
// short scans fill the GPU beside one another instead of one launch (and one
// tail) each.  Each scan is then finalized.  The work buffers that the
// preparation needs only while it runs (raw window, filtered window,
// statistics) are shared by the slots.

struct ScanSlot {
    DeviceBuffer rebin, quads, qscale, image, bp_tables;
    ScanPrep prep;
};

static std::vector<ScanSlot> g_slots;  // the library-wide context's batch slots (its lock)
static DeviceBuffer g_batch_params;

static void swap_slot(Context &c, ScanSlot &sl)
{
    // with FP16 storage the float32 rows are only the filter's input, used
    // while the scan is prepared: one buffer serves every slot
    if (c.storage == 0) std::swap(c.rebin, sl.rebin);
    std::swap(c.quads, sl.quads);
    std::swap(c.qscale, sl.qscale);
    std::swap(c.image, sl.image);
    std::swap(c.bp_tables, sl.bp_tables);
}

static void release_slots()
{
    for (ScanSlot &sl : g_slots) {
        for (DeviceBuffer *b : {&sl.rebin, &sl.quads, &sl.qscale, &sl.image, &sl.bp_tables}) b->release();
    }
    g_slots.clear();
    g_batch_params.release();
}

struct BatchEntry {
    struct recon_metadata *mr;
    float *d_final;
    float mu_water;
};
static std::vector<BatchEntry> g_batch;  // scans added since ctbb_batch_begin (the context's lock)
static std::vector<std::pair<BpShape, BpParams>> g_batch_items;

extern "C" int ctbb_batch_begin(void)
{
    clear_error();
    Context &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    g_batch.clear();
    g_batch_items.clear();
    return CTBB_OK;
}

extern "C" int ctbb_batch_add_device(struct recon_metadata *mr, const float *d_scan, float *d_final, float mu_water)
{
    clear_error();
    if (!mr || !d_scan || !d_final || !mr->table_positions) {
        set_error("ctbb_batch_add_device: metadata not configured or null buffer");
        return CTBB_ERR_ARGUMENT;
    }
    CTBB_TRY(check_mr(mr));
    Context &c = ctx();
    CTBB_TRY(require_device(c));
    std::lock_guard<std::mutex> lk(c.mu);
    return drained(c, [&]() -> int {
        const size_t s = g_batch.size();
        if (g_slots.size() <= s) g_slots.resize(s + 1);
        ScanSlot &sl = g_slots[s];
        swap_slot(c, sl);
        int st = prepare_scan_device(c, mr, d_scan, &sl.prep);
        const size_t plane = (size_t)mr->rp.nx * mr->rp.ny;
        std::vector<std::pair<BpShape, BpParams>> items;
        for (size_t b = 0; st == CTBB_OK && b < sl.prep.blocks.size(); ++b) {
            mr->ri = sl.prep.blocks[b];
            float *slab = c.image.as<float>() + b * mr->ri.n_slices_block * plane;
            const BpShape fallback = window_bp_shape(8, c.storage != 0, sl.prep.tables[b].nht);
            BpParams p;
            BpShape shape = fallback;
            st = prepared_block_params(c, *mr, sl.prep, b, slab, fallback, &p);
            if (st == CTBB_OK) st = tuned_shape(c, p, fallback, &shape);
            if (st == CTBB_OK) st = prepared_block_params(c, *mr, sl.prep, b, slab, shape, &p);
            if (st == CTBB_OK) items.push_back({shape, p});
        }
        swap_slot(c, sl);
        if (st != CTBB_OK) return st;
        g_batch_items.insert(g_batch_items.end(), items.begin(), items.end());
        g_batch.push_back({mr, d_final, mu_water});
        return CTBB_OK;  // drained: d_scan is read to the end when this returns
    });
}

extern "C" int ctbb_batch_run(void)
{
    clear_error();
    Context &c = ctx();
    CTBB_TRY(require_device(c));
    std::lock_guard<std::mutex> lk(c.mu);
    return drained(c, [&]() -> int {
        std::vector<BpShape> shapes;
        for (const auto &it : g_batch_items)
            if (std::find(shapes.begin(), shapes.end(), it.first) == shapes.end()) shapes.push_back(it.first);
        for (const BpShape &sh : shapes) {
            std::vector<BpParams> group;
            for (const auto &it : g_batch_items)
                if (it.first == sh) group.push_back(it.second);
            CTBB_TRY(g_batch_params.ensure(backproject_batch_bytes(group.size())));
            StageScope scope(c, 3);
            CTBB_TRY(launch_backproject_batch(group, sh, g_batch_params.ptr, g_batch_params.bytes, c.stream));
        }
        for (size_t s = 0; s < g_batch.size(); ++s)
            CTBB_TRY(do_finalize(c, *g_batch[s].mr, g_slots[s].image.as<float>(), g_batch[s].d_final,
                                 g_batch[s].mu_water));
        CTBB_CUDA_TRY(cudaStreamSynchronize(c.stream));
        if (c.storage) CTBB_TRY(ramp_tc_check(c.ramp_tc, c.stream));
        g_batch.clear();
        g_batch_items.clear();
        return CTBB_OK;
    });
}

extern "C" int ctbb_reconstruct_batch_device(int n_scans, struct recon_metadata *const *mrs,
                                             const float *const *d_scans, float *const *d_finals, float mu_water)
{
    clear_error();
    if (n_scans <= 0 || !mrs || !d_scans || !d_finals) {
        set_error("ctbb_reconstruct_batch_device: bad argument");
        return CTBB_ERR_ARGUMENT;
    }
    CTBB_TRY(ctbb_batch_begin());
    for (int s = 0; s < n_scans; ++s) {
        int st = ctbb_batch_add_device(mrs[s], d_scans[s], d_finals[s], mu_water);
        if (st != CTBB_OK) {
            std::string err = ctbb_last_error();
            ctbb_batch_begin();
            set_error("scan %d: %s", s, err.c_str());
            return st;
        }
    }
    return ctbb_batch_run();
}

extern "C" int ctbb_set_autotune(int on)
{
    clear_error();
    Context &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    c.autotune = on != 0;
    return CTBB_OK;
}

extern "C" int ctbb_autotune_report(char *buf, size_t n)
{
    std::string out;
    std::vector<BpShape> cq = backproject_shape_candidates(false), cqq = backproject_shape_candidates(true);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (const auto &kv : g_tuned) {
        const TuneKey &k = kv.first;
        const TuneEntry &e = kv.second;
        char line[512];
        int len = snprintf(line, sizeof(line),
                           "%dx%dx%d nos %d rows %d nht %d %s: %s zpt %d threads %d ctas/sm %d cta_w %d;", k.nx, k.ny,
                           k.n_slices, k.nos, k.n_rows, k.nht, k.quad ? "fp16" : "fp32",
                           e.shape.col ? "column" : "tile",
                           e.shape.zpt, e.shape.threads, e.shape.min_blocks, e.shape.cta_w);
        if (e.shape.col) {
            out.append(line, (size_t)std::max(0, std::min(len, (int)sizeof(line) - 1)));
            len = snprintf(line, sizeof(line), " angle chunks %d;", e.shape.achunks);
        }
        out.append(line, (size_t)std::max(0, std::min(len, (int)sizeof(line) - 1)));
        const std::vector<BpShape> &cc = k.quad ? cqq : cq;
        for (int i = 0; i < e.n && i < (int)cc.size(); ++i) {
            if (e.ms[i] <= 0.0) continue;  // not a candidate for this window
            len = snprintf(line, sizeof(line), " %s%d/%d/%d/%dx%d/a%d %.3f ms", cc[i].col ? "c" : "t", cc[i].zpt,
                           cc[i].threads, cc[i].min_blocks, cc[i].cta_w, cc[i].warp_w, cc[i].achunks, e.ms[i]);
            out.append(line, (size_t)std::max(0, std::min(len, (int)sizeof(line) - 1)));
        }
        out += "\n";
    }
    if (buf && n) {
        size_t m = std::min(n - 1, out.size());
        std::memcpy(buf, out.data(), m);
        buf[m] = 0;
    }
    return (int)out.size();
}

extern "C" int ctbb_reconstruct_scan_device(struct recon_metadata *mr, const float *d_scan, float *d_final,
                                            float mu_water)
{
    return reconstruct_scan_device_in(ctx(), mr, d_scan, d_final, mu_water);
}

// --------------------------------------------------------------------------
// drop-in module functions (host buffers)
// --------------------------------------------------------------------------

extern "C" int ctbb_adaptive_filter_kk(struct recon_metadata *mr)
{
    clear_error();
    CTBB_TRY(check_mr(mr));
    if (!mr->ctd.raw) {
        set_error("adaptive_filter_kk: ctd.raw is null");
        return CTBB_ERR_STATE;
    }
    CTBB_TRY(require_device(ctx()));
    Context &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    BlockDims d = block_dims(*mr);
    size_t bytes = d.raw_elems() * sizeof(float);
    CTBB_TRY(c.raw_in.ensure(bytes));
    CTBB_TRY(c.raw_filt.ensure(bytes));
    CTBB_CUDA_TRY(cudaMemcpyAsync(c.raw_in.ptr, mr->ctd.raw, bytes, cudaMemcpyHostToDevice, c.stream));
    CTBB_TRY(do_adaptive(c, *mr, c.raw_in.as<float>(), c.raw_filt.as<float>()));
    CTBB_CUDA_TRY(cudaMemcpyAsync(mr->ctd.raw, c.raw_filt.ptr, bytes, cudaMemcpyDeviceToHost, c.stream));
    CTBB_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return CTBB_OK;
}

extern "C" int ctbb_rebin_filter(struct recon_metadata *mr)
{
    clear_error();
    CTBB_TRY(check_mr(mr));
    if (!mr->ctd.raw) {
        set_error("rebin_filter: ctd.raw is null");
        return CTBB_ERR_STATE;
    }
    CTBB_TRY(require_device(ctx()));
    Context &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    BlockDims d = block_dims(*mr);
    size_t raw_bytes = d.raw_elems() * sizeof(float);
    size_t rebin_bytes = d.rebin_elems() * sizeof(float);
    CTBB_TRY(c.raw_in.ensure(raw_bytes));
    CTBB_CUDA_TRY(cudaMemcpyAsync(c.raw_in.ptr, mr->ctd.raw, raw_bytes, cudaMemcpyHostToDevice, c.stream));
    // d_rebin belongs to the caller until backproject frees it (src/backproject.cu:99);
    // a buffer this library handed out and nobody consumed is released first.
    if (mr->ctd.d_rebin && mr->ctd.d_rebin == c.our_d_rebin) cudaFree(mr->ctd.d_rebin);
    mr->ctd.d_rebin = nullptr;
    float *d_rebin = nullptr;
    CTBB_CUDA_TRY(cudaMalloc(&d_rebin, rebin_bytes));
    mr->ctd.d_rebin = d_rebin;
    c.our_d_rebin = d_rebin;
    CTBB_TRY(do_rebin(c, *mr, c.raw_in.as<float>(), d_rebin));
    CTBB_TRY(do_filter(c, *mr, d_rebin));
    if (mr->flags.testing && mr->ctd.rebin)
        CTBB_CUDA_TRY(cudaMemcpyAsync(mr->ctd.rebin, d_rebin, rebin_bytes, cudaMemcpyDeviceToHost, c.stream));
    CTBB_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return CTBB_OK;
}

extern "C" int ctbb_backproject(struct recon_metadata *mr)
{
    clear_error();
    CTBB_TRY(check_mr(mr));
    if (!mr->ctd.d_rebin || !mr->ctd.image) {
        set_error("backproject: ctd.d_rebin (from rebin_filter) or ctd.image is null");
        return CTBB_ERR_STATE;
    }
    if (mr->ri.cb.block_idx < 1 || (size_t)mr->ri.cb.block_idx > mr->ri.n_blocks) {
        set_error("backproject: block_idx %d outside 1..%zu", mr->ri.cb.block_idx, mr->ri.n_blocks);
        return CTBB_ERR_STATE;
    }
    CTBB_TRY(require_device(ctx()));
    Context &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    size_t plane = (size_t)mr->rp.nx * mr->rp.ny;
    size_t block_elems = plane * mr->ri.n_slices_block;
    CTBB_TRY(c.block.ensure(block_elems * sizeof(float)));
    CTBB_TRY(do_backproject(c, *mr, mr->ctd.d_rebin, c.block.as<float>()));
    size_t block_offset = (size_t)(mr->ri.cb.block_idx - 1) * block_elems;
    CTBB_CUDA_TRY(cudaMemcpyAsync(mr->ctd.image + block_offset, c.block.ptr, block_elems * sizeof(float),
                                  cudaMemcpyDeviceToHost, c.stream));
    CTBB_CUDA_TRY(cudaStreamSynchronize(c.stream));
    CTBB_CUDA_TRY(cudaFree(mr->ctd.d_rebin));
    if (c.our_d_rebin == mr->ctd.d_rebin) c.our_d_rebin = nullptr;
    mr->ctd.d_rebin = nullptr;
    return CTBB_OK;
}

static int finalize_common(struct recon_metadata *mr, float mu_water)
{
    clear_error();
    CTBB_TRY(check_mr(mr));
    if (!mr->ctd.image) {
        set_error("finalize_image_stack: ctd.image is null");
        return CTBB_ERR_STATE;
    }
    if (mr->table_positions && mr->rp.n_readings > 1000) {
        // the slice order follows the table's direction (src/finalize_image_stack_cpu.cu:35)
        double dtp = mr->table_positions[1000] - mr->table_positions[0];
        if (!std::isfinite(dtp) || dtp == 0.0) {
            set_error("finalize_image_stack: table positions 0 and 1000 are equal or not finite (the table "
                      "does not move), so the slice order is undefined");
            return CTBB_ERR_CONFIG;
        }
    }
    CTBB_TRY(require_device(ctx()));
    Context &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    size_t plane = (size_t)mr->rp.nx * mr->rp.ny;
    size_t n_img = plane * mr->ri.n_slices_recon;
    int n_final = ctbb_n_slices_final(mr);
    size_t n_out = plane * (size_t)(n_final > 0 ? n_final : 0);
    CTBB_TRY(c.image.ensure(n_img * sizeof(float)));
    CTBB_TRY(c.final_stack.ensure(n_out * sizeof(float)));
    CTBB_CUDA_TRY(cudaMemcpyAsync(c.image.ptr, mr->ctd.image, n_img * sizeof(float), cudaMemcpyHostToDevice, c.stream));
    CTBB_TRY(do_finalize(c, *mr, c.image.as<float>(), c.final_stack.as<float>(), mu_water));
    float *host = (float *)calloc(n_out ? n_out : 1, sizeof(float));
    if (!host) {
        set_error("finalize_image_stack: host allocation failed");
        return CTBB_ERR_ALLOC;
    }
    CTBB_CUDA_TRY(cudaMemcpyAsync(host, c.final_stack.ptr, n_out * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
    CTBB_CUDA_TRY(cudaStreamSynchronize(c.stream));
    mr->ctd.final_image_stack = host;
    return CTBB_OK;
}

extern "C" int ctbb_finalize_image_stack(struct recon_metadata *mr) { return finalize_common(mr, 0.0f); }

extern "C" int ctbb_finalize_image_stack_hu(struct recon_metadata *mr, float mu_water)
{
    if (!(mu_water > 0.0f)) {
        set_error("finalize_image_stack_hu: mu_water must be > 0");
        return CTBB_ERR_ARGUMENT;
    }
    return finalize_common(mr, mu_water);
}

// C++-linkage drop-ins with the reference module signatures.
int adaptive_filter_kk(struct recon_metadata *mr) { return ctbb_adaptive_filter_kk(mr); }
int rebin_filter(struct recon_metadata *mr) { return ctbb_rebin_filter(mr); }
int backproject(struct recon_metadata *mr) { return ctbb_backproject(mr); }
int finalize_image_stack(struct recon_metadata *mr) { return ctbb_finalize_image_stack(mr); }

// --------------------------------------------------------------------------
// whole scan from host buffers
// --------------------------------------------------------------------------

// the copy stream and the double-buffer events of the host block loop
static int ensure_copy_stream(Context &c)
{
    if (c.copy_stream) return CTBB_OK;
    CTBB_CUDA_TRY(cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking));
    for (int i = 0; i < 2; ++i) {
        CTBB_CUDA_TRY(cudaEventCreateWithFlags(&c.copied[i], cudaEventDisableTiming));
        CTBB_CUDA_TRY(cudaEventCreateWithFlags(&c.consumed[i], cudaEventDisableTiming));
        CTBB_CUDA_TRY(cudaEventRecord(c.consumed[i], c.copy_stream));
    }
    int least = 0, greatest = 0;
    CTBB_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CTBB_CUDA_TRY(cudaStreamCreateWithPriority(&c.prep_stream, cudaStreamNonBlocking, greatest));
    CTBB_CUDA_TRY(cudaEventCreateWithFlags(&c.prep_ready, cudaEventDisableTiming));
    return CTBB_OK;
}

// Enqueues on another stream of the context while in scope: the stage
// helpers take the context's stream, and the streamed path runs its
// preparation on c.prep_stream.  The caller holds c.mu.
struct OnStream {
    Context &c;
    cudaStream_t saved;
    OnStream(Context &cx, cudaStream_t s) : c(cx), saved(cx.stream) { c.stream = s; }
    ~OnStream() { c.stream = saved; }
};

// Where the streamed whole-scan path gets the union window's frames: begin()
// starts the copies of all chunks (each recording chunk_copied[k] on the copy
// stream once its frames are enqueued), issued(k) returns once chunk k's
// copies and event are enqueued, finish() ends any helper thread.
struct ChunkFeed {
    virtual ~ChunkFeed() = default;
    virtual int begin(Context &c, long long g0, long long g1, int chunk, int n_chunks, float *d_raw) = 0;
    virtual int issued(int k) = 0;
    virtual int finish() = 0;
};

// frames [a, e) of the scan from a host array of n_readings frames; frames
// outside [0, n_readings) are zeros
struct HostFeed : ChunkFeed {
    const float *h_scan;
    long long n_readings;
    size_t frame;
    HostFeed(const float *h, long long n, size_t f) : h_scan(h), n_readings(n), frame(f) {}
    int begin(Context &c, long long g0, long long g1, int chunk, int n_chunks, float *d_raw) override
    {
        for (int k = 0; k < n_chunks; ++k) {
            long long a = g0 + (long long)k * chunk, e = std::min(g1, a + chunk);
            long long da = std::max(a, 0LL), de = std::min(e, n_readings);
            float *dst = d_raw + (size_t)(a - g0) * frame;
            if (de <= da) {
                CTBB_CUDA_TRY(cudaMemsetAsync(dst, 0, (size_t)(e - a) * frame * sizeof(float), c.copy_stream));
            } else {
                if (da > a)
                    CTBB_CUDA_TRY(cudaMemsetAsync(dst, 0, (size_t)(da - a) * frame * sizeof(float), c.copy_stream));
                CTBB_CUDA_TRY(cudaMemcpyAsync(d_raw + (size_t)(da - g0) * frame, h_scan + (size_t)da * frame,
                                              (size_t)(de - da) * frame * sizeof(float), cudaMemcpyHostToDevice,
                                              c.copy_stream));
                if (e > de)
                    CTBB_CUDA_TRY(cudaMemsetAsync(d_raw + (size_t)(de - g0) * frame, 0,
                                                  (size_t)(e - de) * frame * sizeof(float), c.copy_stream));
            }
            CTBB_CUDA_TRY(cudaEventRecord(c.chunk_copied[k], c.copy_stream));
        }
        return CTBB_OK;
    }
    int issued(int) override { return CTBB_OK; }
    int finish() override { return CTBB_OK; }
};

// Whole scan, streamed: each chunk of the union window, once its frames are
// on the device, advances the adaptive filter as far as its statistics
// windows allow; the views whose frames are final are rebinned and
// ramp-filtered, and every block whose views are all ready is backprojected.
// Same kernels on the same data as ctbb_reconstruct_scan_device, so the same
// result.  The caller holds c.mu.
static int scan_streamed(Context &c, struct recon_metadata *mr, ChunkFeed &feed, float *h_final, float mu_water)
{
    CTBB_TRY(ensure_copy_stream(c));
    const size_t plane = (size_t)mr->rp.nx * mr->rp.ny;
    const size_t n_block = mr->ri.n_slices_block;
    std::vector<struct recon_info> blocks;
    long long g0 = 0, g1 = 0;
    struct recon_metadata mg;
    CTBB_TRY(plan_union(mr, &blocks, &g0, &g1, &mg));
    BlockDims dg = block_dims(mg);
    const int G = (int)(g1 - g0);
    int n_final = ctbb_n_slices_final(mr);
    size_t max_pull = 0, max_patch = 0, sum_patch = 0;
    edge_extent(*mr, blocks, g0, g1, &max_pull, &max_patch, &sum_patch);
    const size_t af_union = adaptive_filter_scratch_floats(dg.n_proj_pull);
    CTBB_TRY(c.raw_in.ensure(dg.raw_elems() * sizeof(float)));
    CTBB_TRY(c.raw_filt.ensure(dg.raw_elems() * sizeof(float)));
    // the union's rows, then a patch region per block for its re-made edge
    // views (as the device path lays them out): the preparation never waits
    // for a backprojection to free a region, so it runs as far ahead as the
    // frames allow and the host enqueues every block as soon as its rows are
    // ready
    CTBB_TRY(prepare_scan_rows(c, mg, (dg.n_views + sum_patch) * dg.n_rows, dg.n_views * dg.n_rows));
    size_t patch_next = dg.n_views;
    CTBB_TRY(c.scratch.ensure((af_union + adaptive_filter_scratch_floats(max_pull)) * sizeof(float)));
    if (max_patch) {
        CTBB_TRY(c.edge_raw.ensure(max_pull * dg.n_rows_raw * dg.n_channels * sizeof(float)));
        CTBB_TRY(c.dirty.ensure(max_pull));
        if (c.flags_host_bytes < max_pull) {
            if (c.flags_host) cudaFreeHost(c.flags_host);
            c.flags_host = nullptr;
            c.flags_host_bytes = 0;
            CTBB_CUDA_TRY(cudaHostAlloc(reinterpret_cast<void **>(&c.flags_host), max_pull, cudaHostAllocDefault));
            c.flags_host_bytes = max_pull;
        }
        if (!c.flags_ready) CTBB_CUDA_TRY(cudaEventCreateWithFlags(&c.flags_ready, cudaEventDisableTiming));
    }
    CTBB_TRY(c.image.ensure(plane * mr->ri.n_slices_recon * sizeof(float)));
    CTBB_TRY(c.final_stack.ensure(plane * (size_t)(n_final > 0 ? n_final : 1) * sizeof(float)));
    // Two compute streams: the preparation (adaptive filter, rebin, ramp
    // filter, edge flags and patches) on c.prep_stream, the backprojections
    // on the context's stream.  A block's backprojection waits for the
    // preparation enqueued before it (its rows are final); the preparation of
    // later chunks and blocks runs beside it, and neither reading a block's
    // edge flags nor writing its patch waits for a backprojection.  Both
    // start after the work already on the context's stream.
    const cudaStream_t bp_stream = c.stream, prep = c.prep_stream;
    CTBB_CUDA_TRY(cudaEventRecord(c.prep_ready, bp_stream));
    CTBB_CUDA_TRY(cudaStreamWaitEvent(prep, c.prep_ready, 0));
    // the union window in chunks of whole focal-spot cycles; the copy stream
    // starts once the compute streams have finished with the buffer
    const int n_ffs = (int)dg.n_ffs;
    int chunk = (G + scan_chunks() - 1) / scan_chunks();
    chunk = ((chunk + n_ffs - 1) / n_ffs) * n_ffs;
    const int n_chunks = (G + chunk - 1) / chunk;
    while ((int)c.chunk_copied.size() < n_chunks) {
        cudaEvent_t e;
        CTBB_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        c.chunk_copied.push_back(e);
    }
    CTBB_CUDA_TRY(cudaEventRecord(c.consumed[0], prep));
    CTBB_CUDA_TRY(cudaStreamWaitEvent(c.copy_stream, c.consumed[0], 0));
    float *d_raw = c.raw_in.as<float>();
    int status = feed.begin(c, g0, g1, chunk, n_chunks, d_raw);
    // per-scan tables, once
    RebinTables rt;
    if (status == CTBB_OK) status = build_rebin_tables(mg, &rt);
    rt.split_view_coord = 1;  // the union's frame offsets are large
    if (status == CTBB_OK) status = upload_rebin_tables(rt, &c.rebin_tables, prep);
    AfStream af(mg);
    const int V = (int)dg.n_views;
    int v_done = 0;
    size_t b_done = 0;
    for (int k = 0; k < n_chunks && status == CTBB_OK; ++k) {
        status = feed.issued(k);
        if (status != CTBB_OK) break;
        status = cudaStreamWaitEvent(prep, c.chunk_copied[k], 0) == cudaSuccess ? CTBB_OK : CTBB_ERR_CUDA;
        if (status != CTBB_OK) {
            set_error("scan: cudaStreamWaitEvent failed");
            break;
        }
        int arrived = std::min(G, (k + 1) * chunk);
        {
            OnStream on(c, prep);
            {
                StageScope scope(c, 0);
                status = af.advance(mg, d_raw, c.raw_filt.as<float>(), c.scratch.as<float>(), arrived, c.stream);
            }
            if (status != CTBB_OK) break;
            // views whose frames are all final
            int v_ready = V;
            if (af.filtered() < G) {
                v_ready = 0;
                while (v_ready < V && rebin_frames_needed(rt, v_ready) <= af.filtered()) ++v_ready;
            }
            if (v_ready > v_done) {
                {
                    StageScope scope(c, 1);
                    status = launch_rebin(rt, c.rebin_tables, c.raw_filt.as<float>(), c.rebin.as<float>(), c.stream,
                                          v_done, v_ready);
                }
                if (status != CTBB_OK) break;
                status = filter_scan_rows(c, (size_t)v_done * dg.n_rows, (size_t)(v_ready - v_done) * dg.n_rows,
                                          (int)dg.n_rows, (int)dg.n_os);
                if (status != CTBB_OK) break;
                v_done = v_ready;
            }
        }
        // blocks whose views (i + k n_half, k < nht) are all ready, and, for a
        // block with edge views, whose whole window has arrived
        while (b_done < blocks.size() && status == CTBB_OK) {
            struct recon_metadata mb = *mr;
            mb.ri = blocks[b_done];
            BlockDims db = block_dims(mb);
            size_t need = union_view_offset(blocks[b_done], g0) +
                          (size_t)db.n_half_turns * (size_t)(mr->cg.n_proj_turn / 2);
            if (need > (size_t)v_done && v_done < V) break;
            EdgePlan e = edge_plan(mb, g0, g1);
            const long long sb = (long long)(int)blocks[b_done].idx_pull_start - g0;
            // edge views: the union's thresholds of the block's whole window
            if (e.any() && af.filtered() < std::min((long long)G, sb + (long long)db.n_proj_pull)) break;
            mr->ri = blocks[b_done];
            ViewRows vr;
            vr.off = union_view_offset(blocks[b_done], g0);
            vr.patch = patch_next;
            patch_next += (size_t)e.n_patch();
            if (e.any()) {
                OnStream on(c, prep);
                float *d_block_scratch = c.scratch.as<float>() + af_union;
                status = edge_dirty_frames(c, mb, e, d_raw, c.scratch.as<float>(),
                                           c.scratch.as<float>() + 5 * (size_t)dg.n_proj_pull, g0, g1,
                                           d_block_scratch, c.dirty.as<unsigned char>());
                if (status == CTBB_OK &&
                    (cudaMemcpyAsync(c.flags_host, c.dirty.ptr, db.n_proj_pull, cudaMemcpyDeviceToHost, prep) !=
                         cudaSuccess ||
                     cudaEventRecord(c.flags_ready, prep) != cudaSuccess ||
                     cudaEventSynchronize(c.flags_ready) != cudaSuccess)) {
                    set_error("whole scan: reading the edge frames' flags failed");
                    status = CTBB_ERR_CUDA;
                }
                if (status != CTBB_OK) break;
                const auto runs = dirty_view_runs(e, block_rebin_tables(rt, db), c.flags_host, (int)db.n_proj_pull);
                vr.slot.assign((size_t)e.n_used, -1);
                size_t made = 0;
                status = run_edge_patch(c, mb, rt, runs, d_raw, c.scratch.as<float>(), g0, d_block_scratch,
                                        vr.patch, &vr, &made);
            }
            if (status != CTBB_OK) break;
            if (cudaEventRecord(c.prep_ready, prep) != cudaSuccess ||
                cudaStreamWaitEvent(bp_stream, c.prep_ready, 0) != cudaSuccess) {
                set_error("scan: ordering the backprojection after its rows failed");
                status = CTBB_ERR_CUDA;
                break;
            }
            float *slab = c.image.as<float>() + b_done * n_block * plane;
            status = backproject_scan_rows(c, *mr, slab, vr);
            ++b_done;
        }
    }
    int fs = feed.finish();
    if (status != CTBB_OK) return status;
    if (fs != CTBB_OK) return fs;
    if (b_done != blocks.size()) {
        set_error("whole scan: %zu of %zu blocks left unfinished", blocks.size() - b_done, blocks.size());
        return CTBB_ERR_STATE;
    }
    // the last backprojection waited for all the preparation: the tensor-core
    // filter's error flag is final on the context's stream too
    CTBB_TRY(do_finalize(c, *mr, c.image.as<float>(), c.final_stack.as<float>(), mu_water));
    CTBB_CUDA_TRY(cudaMemcpyAsync(h_final, c.final_stack.ptr, plane * (size_t)n_final * sizeof(float),
                                  cudaMemcpyDeviceToHost, c.stream));
    if (c.storage) CTBB_TRY(ramp_tc_check(c.ramp_tc, c.stream));
    CTBB_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return CTBB_OK;
}

// Whole scan from host buffers, streamed: the union window is copied in
// chunks on the copy stream while the compute stream works on the chunks
// that have arrived (scan_streamed).  Same result as
// ctbb_reconstruct_scan_device.
static int reconstruct_scan_host_in(Context &c, struct recon_metadata *mr, const float *h_scan, float *h_final,
                                          float mu_water)
{
    clear_error();
    if (!mr || !h_scan || !h_final || !mr->table_positions) {
        set_error("ctbb_reconstruct_scan_host: metadata not configured or null buffer");
        return CTBB_ERR_ARGUMENT;
    }
    CTBB_TRY(check_mr(mr));
    CTBB_TRY(require_device(c));
    std::lock_guard<std::mutex> lk(c.mu);
    return drained(c, [&]() -> int {
        HostFeed feed(h_scan, (long long)mr->rp.n_readings, mr->cg.n_rows_raw * mr->cg.n_channels);
        return scan_streamed(c, mr, feed, h_final, mu_water);
    });
}

extern "C" int ctbb_reconstruct_scan_host(struct recon_metadata *mr, const float *h_scan, float *h_final,
                                          float mu_water)
{
    return reconstruct_scan_host_in(ctx(), mr, h_scan, h_final, mu_water);
}

// Frames [a, e) of the scan read from a FileType 0 raw file -- frame i at
// byte raw_data_offset + i * frame_bytes, frames before the start or past the
// end of the file read as zeros, as extract_projections reads them.  A reader
// thread fills two pinned staging buffers in turn and enqueues each chunk's
// host->device copy itself, so the copies never wait for the compute loop.
constexpr int kReadThreads = 8;  // threads reading one chunk of the raw file

struct FileFeed : ChunkFeed {
    std::string path;
    long long offset;
    size_t frame;
    std::thread reader;
    std::mutex mu;
    std::condition_variable cv;
    int n_issued = 0;
    bool stop = false;  // set by finish(): no further chunks
    int status = CTBB_OK;
    std::string error;
    FileFeed(std::string p, long long off, size_t f) : path(std::move(p)), offset(off), frame(f) {}
    ~FileFeed() override
    {
        if (reader.joinable()) reader.join();
    }
    void fail(const char *what)
    {
        std::lock_guard<std::mutex> lk(mu);
        if (status == CTBB_OK) {
            status = CTBB_ERR_IO;
            error = what;
        }
        cv.notify_all();
    }
    int begin(Context &c, long long g0, long long g1, int chunk, int n_chunks, float *d_raw) override
    {
        const size_t need = (size_t)chunk * frame * sizeof(float);
        if (c.stage_bytes < need) {
            for (int i = 0; i < 2; ++i) {
                if (c.stage[i]) cudaFreeHost(c.stage[i]);
                c.stage[i] = nullptr;
            }
            c.stage_bytes = 0;
            for (int i = 0; i < 2; ++i) CTBB_CUDA_TRY(cudaHostAlloc(&c.stage[i], need, cudaHostAllocDefault));
            c.stage_bytes = need;
        }
        for (int i = 0; i < 2; ++i) {
            if (!c.stage_free[i]) CTBB_CUDA_TRY(cudaEventCreateWithFlags(&c.stage_free[i], cudaEventDisableTiming));
            CTBB_CUDA_TRY(cudaEventRecord(c.stage_free[i], c.copy_stream));
        }
        int fd = open(path.c_str(), O_RDONLY);
        if (fd < 0) {
            set_error("raw data file %s not found", path.c_str());
            return CTBB_ERR_IO;
        }
        int dev = 0;
        CTBB_CUDA_TRY(cudaGetDevice(&dev));
        reader = std::thread([this, &c, fd, g0, g1, chunk, n_chunks, d_raw, dev] {
            cudaSetDevice(dev);
            for (int k = 0; k < n_chunks; ++k) {
                {
                    std::lock_guard<std::mutex> lk(mu);
                    if (stop || status != CTBB_OK) break;
                }
                int slot = k & 1;
                if (cudaEventSynchronize(c.stage_free[slot]) != cudaSuccess) {
                    fail("staging buffer wait failed");
                    break;
                }
                long long a = g0 + (long long)k * chunk, e = std::min(g1, a + chunk);
                float *stage = static_cast<float *>(c.stage[slot]);
                size_t n = (size_t)(e - a) * frame;
                long long ra = std::max(a, 0LL);
                if (ra > a) memset(stage, 0, (size_t)(ra - a) * frame * sizeof(float));  // before frame 0
                if (e > ra) read_frames(fd, offset + ra * (long long)(frame * sizeof(float)),
                                        reinterpret_cast<char *>(stage + (size_t)(ra - a) * frame),
                                        (size_t)(e - ra) * frame * sizeof(float));
                if (cudaMemcpyAsync(d_raw + (size_t)(a - g0) * frame, stage, n * sizeof(float),
                                    cudaMemcpyHostToDevice, c.copy_stream) != cudaSuccess ||
                    cudaEventRecord(c.stage_free[slot], c.copy_stream) != cudaSuccess ||
                    cudaEventRecord(c.chunk_copied[k], c.copy_stream) != cudaSuccess) {
                    fail("host->device copy of a raw chunk failed");
                    break;
                }
                std::lock_guard<std::mutex> lk(mu);
                n_issued = k + 1;
                cv.notify_all();
            }
            close(fd);
        });
        return CTBB_OK;
    }
    // bytes [pos, pos + len) of the file into dst by several threads at once;
    // what lies past the end of the file reads as zeros
    static void read_frames(int fd, long long pos, char *dst, size_t len)
    {
        const size_t kSlice = (size_t)32 << 20;
        size_t n_slices = (len + kSlice - 1) / kSlice;
        int n_threads = (int)std::min<size_t>(n_slices, (size_t)kReadThreads);
        std::atomic<size_t> next{0};
        auto work = [&] {
            for (size_t i = next++; i < n_slices; i = next++) {
                size_t off = i * kSlice, want = std::min(kSlice, len - off), got = 0;
                while (got < want) {
                    ssize_t r = pread(fd, dst + off + got, want - got, (off_t)(pos + (long long)(off + got)));
                    if (r <= 0) break;
                    got += (size_t)r;
                }
                if (got < want) memset(dst + off + got, 0, want - got);
            }
        };
        std::vector<std::thread> pool;
        for (int t = 1; t < n_threads; ++t) pool.emplace_back(work);
        work();
        for (auto &t : pool) t.join();
    }
    int issued(int k) override
    {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return n_issued > k || status != CTBB_OK; });
        if (n_issued > k) return CTBB_OK;
        set_error("%s", error.c_str());
        return status;
    }
    int finish() override
    {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;  // the compute loop is done with the chunks (or gave up)
        }
        if (reader.joinable()) reader.join();
        std::lock_guard<std::mutex> lk(mu);
        if (status != CTBB_OK) set_error("%s", error.c_str());
        return status;
    }
};

// Whole scan straight from the raw file (FileType 0): the file is read in
// chunks while earlier chunks are copied and processed (scan_streamed).
// Same result as ctbb_reconstruct_scan_device on the file's frames.
static int reconstruct_scan_file_in(Context &c, struct recon_metadata *mr, float *h_final, float mu_water)
{
    clear_error();
    if (!mr || !h_final || !mr->table_positions) {
        set_error("ctbb_reconstruct_scan_file: metadata not configured or null buffer");
        return CTBB_ERR_ARGUMENT;
    }
    if (mr->rp.file_type != 0) {
        set_error("ctbb_reconstruct_scan_file: FileType %d is not read here (only 0, float32 frames)",
                  mr->rp.file_type);
        return CTBB_ERR_CONFIG;
    }
    CTBB_TRY(check_mr(mr));
    CTBB_TRY(require_device(c));
    std::lock_guard<std::mutex> lk(c.mu);
    return drained(c, [&]() -> int {
        char path[4096 + 255 + 2];
        snprintf(path, sizeof(path), "%s/%s", mr->rp.raw_data_dir, mr->rp.raw_data_file);
        FileFeed feed(path, (long long)mr->rp.raw_data_offset, mr->cg.n_rows_raw * mr->cg.n_channels);
        return scan_streamed(c, mr, feed, h_final, mu_water);
    });
}

extern "C" int ctbb_reconstruct_scan_file(struct recon_metadata *mr, float *h_final, float mu_water)
{
    return reconstruct_scan_file_in(ctx(), mr, h_final, mu_water);
}

static int reconstruct_host_in(Context &c, struct recon_metadata *mr, const float *h_scan, float *h_final,
                                     float mu_water)
{
    clear_error();
    if (!mr || !h_scan || !h_final || !mr->table_positions) {
        set_error("ctbb_reconstruct_host: metadata not configured or null buffer");
        return CTBB_ERR_ARGUMENT;
    }
    CTBB_TRY(check_mr(mr));
    CTBB_TRY(require_device(c));
    std::lock_guard<std::mutex> lk(c.mu);
    return drained(c, [&]() -> int {
        CTBB_TRY(ensure_copy_stream(c));
        const size_t frame = mr->cg.n_rows_raw * mr->cg.n_channels;
        const long long n_readings = mr->rp.n_readings;
        const size_t plane = (size_t)mr->rp.nx * mr->rp.ny;
        const size_t n_block = mr->ri.n_slices_block;
        CTBB_TRY(c.image.ensure(plane * mr->ri.n_slices_recon * sizeof(float)));
        int n_final = ctbb_n_slices_final(mr);
        CTBB_TRY(c.final_stack.ensure(plane * (size_t)(n_final > 0 ? n_final : 1) * sizeof(float)));
        DeviceBuffer *win[2] = {&c.raw_in, &c.raw_in2};
        mr->ri.cb.block_idx = 0;
        for (size_t b = 0; b < mr->ri.n_blocks; ++b) {
            struct recon_info ri;
            CTBB_TRY(plan_next_block(*mr, &ri));
            mr->ri = ri;
            BlockDims d = block_dims(*mr);
            int slot = (int)(b & 1);
            CTBB_TRY(win[slot]->ensure(d.raw_elems() * sizeof(float)));
            // H2D of the block's window on the copy stream, once the buffer's
            // previous reader (the adaptive filter two blocks back) is done
            CTBB_CUDA_TRY(cudaStreamWaitEvent(c.copy_stream, c.consumed[slot], 0));
            long long s0 = (long long)(int)mr->ri.idx_pull_start, s1 = s0 + (long long)d.n_proj_pull;
            long long a = s0 < 0 ? 0 : s0, e = s1 > n_readings ? n_readings : s1;
            float *dst = win[slot]->as<float>();
            if (a > s0) CTBB_CUDA_TRY(cudaMemsetAsync(dst, 0, (size_t)(a - s0) * frame * sizeof(float), c.copy_stream));
            if (e < s1) {
                long long z0 = e > s0 ? e : s0;
                CTBB_CUDA_TRY(cudaMemsetAsync(dst + (size_t)(z0 - s0) * frame, 0, (size_t)(s1 - z0) * frame * sizeof(float),
                                              c.copy_stream));
            }
            if (e > a)
                CTBB_CUDA_TRY(cudaMemcpyAsync(dst + (size_t)(a - s0) * frame, h_scan + (size_t)a * frame,
                                              (size_t)(e - a) * frame * sizeof(float), cudaMemcpyHostToDevice,
                                              c.copy_stream));
            CTBB_CUDA_TRY(cudaEventRecord(c.copied[slot], c.copy_stream));
            CTBB_CUDA_TRY(cudaStreamWaitEvent(c.stream, c.copied[slot], 0));
            CTBB_TRY(c.raw_filt.ensure(d.raw_elems() * sizeof(float)));
            CTBB_TRY(do_adaptive(c, *mr, dst, c.raw_filt.as<float>()));
            CTBB_CUDA_TRY(cudaEventRecord(c.consumed[slot], c.stream));
            CTBB_TRY(c.rebin.ensure(d.rebin_elems() * sizeof(float)));
            CTBB_TRY(do_rebin(c, *mr, c.raw_filt.as<float>(), c.rebin.as<float>()));
            CTBB_TRY(do_filter(c, *mr, c.rebin.as<float>()));
            CTBB_TRY(do_backproject(c, *mr, c.rebin.as<float>(), c.image.as<float>() + b * n_block * plane));
        }
        CTBB_TRY(do_finalize(c, *mr, c.image.as<float>(), c.final_stack.as<float>(), mu_water));
        CTBB_CUDA_TRY(cudaMemcpyAsync(h_final, c.final_stack.ptr, plane * (size_t)n_final * sizeof(float),
                                      cudaMemcpyDeviceToHost, c.stream));
        CTBB_CUDA_TRY(cudaStreamSynchronize(c.stream));
        return CTBB_OK;
    });
}

extern "C" int ctbb_reconstruct_host(struct recon_metadata *mr, const float *h_scan, float *h_final,
                                     float mu_water)
{
    return reconstruct_host_in(ctx(), mr, h_scan, h_final, mu_water);
}

// --------------------------------------------------------------------------
// per-stage timing
// --------------------------------------------------------------------------

extern "C" int ctbb_profile_enable(int on)
{
    Context &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    c.profiling = on != 0;
    return CTBB_OK;
}

extern "C" int ctbb_profile_read(double *ms, uint64_t *launches, int n, int reset)
{
    clear_error();
    Context &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    for (int s = 0; s < kProfileStages; ++s) {
        for (auto &ev : c.open_events[s]) {
            CTBB_CUDA_TRY(cudaEventSynchronize(ev.second));
            float t = 0.0f;
            CTBB_CUDA_TRY(cudaEventElapsedTime(&t, ev.first, ev.second));
            c.stage_ms[s] += t;
            c.stage_launches[s] += 1;
            c.event_pool.push_back(ev.first);
            c.event_pool.push_back(ev.second);
        }
        c.open_events[s].clear();
    }
    for (int s = 0; s < n && s < kProfileStages; ++s) {
        if (ms) ms[s] = c.stage_ms[s];
        if (launches) launches[s] = c.stage_launches[s];
    }
    if (reset)
        for (int s = 0; s < kProfileStages; ++s) {
            c.stage_ms[s] = 0.0;
            c.stage_launches[s] = 0;
        }
    return kProfileStages;
}

// --------------------------------------------------------------------------
// contexts: independent work buffers and streams for concurrent scans
// --------------------------------------------------------------------------

struct ctbb_context_s {
    Context c;
    bool own_stream = false;
};

static size_t context_device_bytes(const Context &c)
{
    size_t n = 0;
    for (const DeviceBuffer *b : {&c.raw_in, &c.raw_in2, &c.raw_filt, &c.rebin, &c.block, &c.image, &c.final_stack,
                                  &c.scratch, &c.bp_views, &c.bp_theta, &c.bp_zpos, &c.fin_offsets, &c.fin_slices,
                                  &c.fin_weights, &c.edge_raw, &c.dirty, &c.tc_work, &c.quads, &c.qscale,
                                  &c.bp_tables, &c.bp_partial})
        n += b->bytes;
    return n + c.ramp.capacity * sizeof(float2);
}

extern "C" int ctbb_context_create(ctbb_context *out)
{
    clear_error();
    if (!out) {
        set_error("ctbb_context_create: null argument");
        return CTBB_ERR_ARGUMENT;
    }
    *out = nullptr;
    ctbb_context h = new (std::nothrow) ctbb_context_s;
    if (!h) {
        set_error("ctbb_context_create: out of host memory");
        return CTBB_ERR_ALLOC;
    }
    int st = require_device(h->c);
    if (st == CTBB_OK && cudaStreamCreateWithFlags(&h->c.stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("ctbb_context_create: cudaStreamCreateWithFlags failed");
        st = CTBB_ERR_CUDA;
    }
    if (st != CTBB_OK) {
        delete h;
        return st;
    }
    h->own_stream = true;
    *out = h;
    return CTBB_OK;
}

extern "C" int ctbb_context_destroy(ctbb_context h)
{
    clear_error();
    if (!h) return CTBB_OK;
    {
        std::lock_guard<std::mutex> lk(h->c.mu);
        release_context(h->c, false, false);
        if (h->own_stream && h->c.stream) cudaStreamDestroy(h->c.stream);
        h->c.stream = nullptr;
        for (cudaEvent_t e : h->c.event_pool) cudaEventDestroy(e);
        h->c.event_pool.clear();
    }
    delete h;
    return CTBB_OK;
}

extern "C" int ctbb_context_set_storage(ctbb_context h, int mode)
{
    clear_error();
    if (!h) {
        set_error("ctbb_context_set_storage: null context");
        return CTBB_ERR_ARGUMENT;
    }
    return set_storage(h->c, mode);
}

extern "C" int ctbb_context_set_stream(ctbb_context h, void *stream)
{
    clear_error();
    if (!h) {
        set_error("ctbb_context_set_stream: null context");
        return CTBB_ERR_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(h->c.mu);
    cudaStreamSynchronize(h->c.stream);
    if (h->own_stream && h->c.stream) cudaStreamDestroy(h->c.stream);
    h->own_stream = false;
    h->c.stream = reinterpret_cast<cudaStream_t>(stream);
    return CTBB_OK;
}

extern "C" int ctbb_context_release_workspace(ctbb_context h)
{
    clear_error();
    if (!h) {
        set_error("ctbb_context_release_workspace: null context");
        return CTBB_ERR_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(h->c.mu);
    release_context(h->c, false, false);
    return CTBB_OK;
}

extern "C" size_t ctbb_context_device_bytes(ctbb_context h)
{
    if (!h) return 0;
    std::lock_guard<std::mutex> lk(h->c.mu);
    return context_device_bytes(h->c);
}

#define CTBB_CONTEXT_CALL(h, impl, ...)                                   \
    do {                                                                  \
        if (!(h)) {                                                       \
            clear_error();                                                \
            set_error("%s: null context", __func__);                      \
            return CTBB_ERR_ARGUMENT;                                     \
        }                                                                 \
        return impl((h)->c, __VA_ARGS__);                                 \
    } while (0)

extern "C" int ctbb_context_reconstruct_scan_device(ctbb_context h, struct recon_metadata *mr, const float *d_scan,
                                                    float *d_final, float mu_water)
{
    CTBB_CONTEXT_CALL(h, reconstruct_scan_device_in, mr, d_scan, d_final, mu_water);
}

extern "C" int ctbb_context_reconstruct_scan_host(ctbb_context h, struct recon_metadata *mr, const float *h_scan,
                                                  float *h_final, float mu_water)
{
    CTBB_CONTEXT_CALL(h, reconstruct_scan_host_in, mr, h_scan, h_final, mu_water);
}

extern "C" int ctbb_context_reconstruct_scan_file(ctbb_context h, struct recon_metadata *mr, float *h_final,
                                                  float mu_water)
{
    CTBB_CONTEXT_CALL(h, reconstruct_scan_file_in, mr, h_final, mu_water);
}

extern "C" int ctbb_context_reconstruct_device(ctbb_context h, struct recon_metadata *mr, const float *d_scan,
                                               float *d_final, float mu_water)
{
    CTBB_CONTEXT_CALL(h, reconstruct_device_in, mr, d_scan, d_final, mu_water);
}

extern "C" int ctbb_context_reconstruct_host(ctbb_context h, struct recon_metadata *mr, const float *h_scan,
                                             float *h_final, float mu_water)
{
    CTBB_CONTEXT_CALL(h, reconstruct_host_in, mr, h_scan, h_final, mu_water);
}

// phantom.cu -- analytic forward projector for seeded helical phantoms.
//
// Produces the raw input of the hot path (test and benchmark data; the
// reference ships no raw data).  Test infrastructure: built into
// libctbb_synth.so, not into the reconstruction library.  The geometry is the one the reference's
// rebinning and backprojection invert:
//
//  * frame f: nominal source angle phi_f = tube_angles[f] (deg) and source z =
//    table_positions[f]; its focal spot is f mod n_ffs with the offsets of
//    src/rebin_filter_cpu.cu:161-645 -- phi-FFS (+da, -da), z-FFS (-dr, +dr),
//    both: (+da,-dr), (-da,-dr), (+da,+dr), (-da,+dr).  In the rotating frame
//    (u toward the nominal source, v = u rotated by +90 deg) the focal spot sits
//    at (r_f + dr, da) and dr*tan(anode) above the nominal source z, with
//    da = D r_f fai / (4 (D - r_f)), dr = D coll / (4 (D - r_f) tan(anode));
//  * channel ch: detector arc of radius D centred on the nominal focal spot,
//    element at (r_f - D cos b, -D sin b), b = (ch - central_channel) * fai
//    (beta_rk, src/rebin_filter_cpu.cu:41-44);
//  * raw row r: height (r - (R_raw - 1)/2) * coll * D / r_f above the nominal
//    source z (row slope tan(theta_cone/2) (2r/(R-1) - 1) of the backprojector,
//    src/backproject_cpu.cu:112-113).
//
// Line integrals are exact chords through infinite z-cylinders and rotated
// ellipsoids (attenuations add).  Optional Poisson noise: counts drawn from a
// counter-based generator keyed by (seed, frame, row, channel), so any frame
// range and the host/device variants agree up to libm rounding.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "synth.h"

namespace synth {

namespace {
thread_local char g_error[512] = "";
}

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
}

constexpr int kMaxPhantomObjects = 128;

struct PhantomScan {
    float r_f, src_to_det, fai, cc, coll, tan_anode;
    float da, dr;
    int n_channels, n_rows_raw, n_ffs, phi_ffs, z_ffs;
    int n_objects;
    float i0;
    unsigned long long seed;
    ctbb_phantom_object obj[kMaxPhantomObjects];
};

__host__ __device__ inline unsigned long long mix64(unsigned long long z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// uniform in (0, 1]
__host__ __device__ inline float uniform01(unsigned long long key, unsigned int k)
{
    unsigned long long h = mix64(key ^ mix64(0x5851F42D4C957F2Dull * (k + 1)));
    return ((float)(h >> 40) + 1.0f) * (1.0f / 16777216.0f);
}

__host__ __device__ inline float poisson_draw(float lambda, unsigned long long key)
{
    if (lambda > 30.0f) {
        float u1 = uniform01(key, 0), u2 = uniform01(key, 1);
        float g = sqrtf(-2.0f * logf(u1)) * cosf(6.28318530718f * u2);
        float n = floorf(lambda + sqrtf(lambda) * g + 0.5f);
        return n < 0.0f ? 0.0f : n;
    }
    // Knuth's product-of-uniforms method; at most 200 draws (lambda <= 30).
    float limit = expf(-lambda), prod = 1.0f;
    int k = 0;
    for (; k < 200; ++k) {
        prod *= uniform01(key, 2 + k);
        if (prod <= limit) break;
    }
    return (float)k;
}

// focal-spot offsets (da, dr) of focal position q (frame mod n_ffs)
__host__ __device__ inline void focal_offsets(const PhantomScan &s, int q, float *da, float *dr)
{
    *da = 0.0f;
    *dr = 0.0f;
    if (s.phi_ffs && s.z_ffs) {
        *da = (q & 1) ? -s.da : s.da;
        *dr = (q & 2) ? s.dr : -s.dr;
    } else if (s.phi_ffs) {
        *da = (q & 1) ? -s.da : s.da;
    } else if (s.z_ffs) {
        *dr = (q & 1) ? s.dr : -s.dr;
    }
}

// Sum of mu * chord over the segment a -> b.
__host__ __device__ inline float line_integral(const PhantomScan &s, const float a[3],
                                               const float b[3])
{
    float d[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    float len = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    float total = 0.0f;
    for (int o = 0; o < s.n_objects; ++o) {
        const ctbb_phantom_object &ob = s.obj[o];
        float t_in, t_out;
        if (ob.kind == 0) {
            // infinite cylinder along z: |(a + t d)_xy - c_xy| = R
            float ox = a[0] - ob.center[0], oy = a[1] - ob.center[1];
            float A = d[0] * d[0] + d[1] * d[1];
            float B = ox * d[0] + oy * d[1];
            float Cc = ox * ox + oy * oy - ob.semi_axes[0] * ob.semi_axes[0];
            float disc = B * B - A * Cc;
            if (A <= 0.0f || disc <= 0.0f) continue;
            float sq = sqrtf(disc);
            t_in = (-B - sq) / A;
            t_out = (-B + sq) / A;
        } else {
            float o3[3] = {a[0] - ob.center[0], a[1] - ob.center[1], a[2] - ob.center[2]};
            float ob3[3], db3[3];
            for (int r = 0; r < 3; ++r) {
                ob3[r] = (ob.rotation[3 * r] * o3[0] + ob.rotation[3 * r + 1] * o3[1] +
                          ob.rotation[3 * r + 2] * o3[2]) / ob.semi_axes[r];
                db3[r] = (ob.rotation[3 * r] * d[0] + ob.rotation[3 * r + 1] * d[1] +
                          ob.rotation[3 * r + 2] * d[2]) / ob.semi_axes[r];
            }
            float A = db3[0] * db3[0] + db3[1] * db3[1] + db3[2] * db3[2];
            float B = ob3[0] * db3[0] + ob3[1] * db3[1] + ob3[2] * db3[2];
            float Cc = ob3[0] * ob3[0] + ob3[1] * ob3[1] + ob3[2] * ob3[2] - 1.0f;
            float disc = B * B - A * Cc;
            if (A <= 0.0f || disc <= 0.0f) continue;
            float sq = sqrtf(disc);
            t_in = (-B - sq) / A;
            t_out = (-B + sq) / A;
        }
        t_in = fmaxf(t_in, 0.0f);
        t_out = fminf(t_out, 1.0f);
        if (t_out > t_in) total += ob.mu * (t_out - t_in) * len;
    }
    return total;
}

__host__ __device__ inline float project_sample(const PhantomScan &s, size_t frame, float angle_deg,
                                                double table_pos, int row, int ch)
{
    int q = (int)(frame % (size_t)s.n_ffs);
    float da, dr;
    focal_offsets(s, q, &da, &dr);
    float phi = angle_deg * (3.14159265358979f / 180.0f);
    float cp = cosf(phi), sp = sinf(phi);
    float zs = (float)table_pos;
    // focal spot and detector element in the rotating frame (u, v, z)
    float fu = s.r_f + dr, fv = da, fz = zs + dr * s.tan_anode;
    float b = ((float)ch - s.cc) * s.fai;
    float pu = s.r_f - s.src_to_det * cosf(b), pv = -s.src_to_det * sinf(b);
    float pz = zs + ((float)row - 0.5f * (float)(s.n_rows_raw - 1)) * s.coll * s.src_to_det / s.r_f;
    float a3[3] = {fu * cp - fv * sp, fu * sp + fv * cp, fz};
    float b3[3] = {pu * cp - pv * sp, pu * sp + pv * cp, pz};
    float p = line_integral(s, a3, b3);
    if (s.i0 > 0.0f) {
        unsigned long long key =
            mix64(s.seed ^ mix64(((unsigned long long)frame << 24) ^
                                 ((unsigned long long)row << 12) ^ (unsigned long long)ch));
        float n = poisson_draw(s.i0 * expf(-p), key);
        p = -logf(fmaxf(n, 1.0f) / s.i0);
    }
    return p;
}

__global__ void phantom_project_kernel(const PhantomScan *__restrict__ scan,
                                       const float *__restrict__ tube_angles,
                                       const double *__restrict__ table_positions,
                                       size_t n_readings, size_t frame0, size_t n_frames,
                                       float *__restrict__ out)
{
    const PhantomScan &s = *scan;
    size_t per_frame = (size_t)s.n_channels * s.n_rows_raw;
    size_t total = per_frame * n_frames;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        size_t fl = i / per_frame;
        size_t rem = i - fl * per_frame;
        int row = (int)(rem / s.n_channels);
        int ch = (int)(rem - (size_t)row * s.n_channels);
        size_t frame = frame0 + fl;
        float v = 0.0f;
        if (frame < n_readings) v = project_sample(s, frame, tube_angles[frame],
                                                   table_positions[frame], row, ch);
        out[i] = v;
    }
}

static int make_scan(const struct recon_metadata *mr, const ctbb_phantom_object *objects,
                     int n_objects, float i0, unsigned long long seed, PhantomScan *s)
{
    if (!mr || (!objects && n_objects) || n_objects < 0 || n_objects > kMaxPhantomObjects) {
        set_error("phantom: bad arguments (at most %d objects)", kMaxPhantomObjects);
        return 1;
    }
    const struct ct_geom &cg = mr->cg;
    memset(s, 0, sizeof(*s));
    s->r_f = cg.r_f;
    s->src_to_det = cg.src_to_det;
    s->fai = cg.fan_angle_increment;
    s->cc = cg.central_channel;
    s->coll = mr->rp.coll_slicewidth;
    s->tan_anode = tanf(cg.anode_angle);
    s->da = cg.src_to_det * cg.r_f * cg.fan_angle_increment / (4.0f * (cg.src_to_det - cg.r_f));
    s->dr = (float)(cg.src_to_det * mr->rp.coll_slicewidth /
                    (4.0 * (cg.src_to_det - cg.r_f) * tanf(cg.anode_angle)));
    s->n_channels = (int)cg.n_channels;
    s->n_rows_raw = (int)cg.n_rows_raw;
    s->phi_ffs = mr->rp.phi_ffs ? 1 : 0;
    s->z_ffs = mr->rp.z_ffs ? 1 : 0;
    s->n_ffs = 1 << (s->phi_ffs + s->z_ffs);
    s->n_objects = n_objects;
    s->i0 = i0;
    s->seed = seed;
    if (n_objects) memcpy(s->obj, objects, sizeof(ctbb_phantom_object) * (size_t)n_objects);
    if (s->n_channels <= 0 || s->n_rows_raw <= 0) {
        set_error("phantom: geometry not configured");
        return 8;
    }
    return 0;
}

}  // namespace synth

using namespace synth;

extern "C" const char *synth_last_error(void) { return g_error; }

extern "C" int synth_project_host(const struct recon_metadata *mr, const struct ctbb_phantom_object *objects,
                                  int n_objects, size_t frame0, size_t n_frames, float i0, uint64_t seed,
                                  float *out)
{
    g_error[0] = 0;
    PhantomScan *s = new PhantomScan;
    int st = make_scan(mr, objects, n_objects, i0, seed, s);
    if (st) {
        delete s;
        return st;
    }
    if (!out || !mr->tube_angles || !mr->table_positions) {
        delete s;
        set_error("phantom: null output or frame tables");
        return 1;
    }
    size_t n_readings = (size_t)mr->rp.n_readings;
    size_t per_frame = (size_t)s->n_channels * s->n_rows_raw;
    for (size_t fl = 0; fl < n_frames; ++fl) {
        size_t frame = frame0 + fl;
        for (int row = 0; row < s->n_rows_raw; ++row)
            for (int ch = 0; ch < s->n_channels; ++ch) {
                float v = 0.0f;
                if (frame < n_readings)
                    v = project_sample(*s, frame, mr->tube_angles[frame],
                                       mr->table_positions[frame], row, ch);
                out[fl * per_frame + (size_t)row * s->n_channels + ch] = v;
            }
    }
    delete s;
    return 0;
}

#define SYNTH_CUDA_TRY(expr)                                                          \
    do {                                                                              \
        cudaError_t e_ = (expr);                                                      \
        if (e_ != cudaSuccess) {                                                      \
            set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return 5;                                                                 \
        }                                                                             \
    } while (0)

extern "C" int synth_project_device(const struct recon_metadata *mr, const struct ctbb_phantom_object *objects,
                                    int n_objects, const float *d_tube_angles, const double *d_table_positions,
                                    size_t frame0, size_t n_frames, float i0, uint64_t seed, float *d_out,
                                    void *stream_ptr)
{
    g_error[0] = 0;
    if (!d_out || !d_tube_angles || !d_table_positions) {
        set_error("phantom: null device pointer");
        return 1;
    }
    std::vector<char> host(sizeof(PhantomScan));
    PhantomScan *s = reinterpret_cast<PhantomScan *>(host.data());
    int st = make_scan(mr, objects, n_objects, i0, seed, s);
    if (st) return st;
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_ptr);
    int dev = 0, sms = 0;
    SYNTH_CUDA_TRY(cudaGetDevice(&dev));
    SYNTH_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PhantomScan *d_scan = nullptr;
    SYNTH_CUDA_TRY(cudaMallocAsync((void **)&d_scan, sizeof(PhantomScan), stream));
    SYNTH_CUDA_TRY(cudaMemcpyAsync(d_scan, s, sizeof(PhantomScan), cudaMemcpyHostToDevice, stream));
    size_t total = (size_t)s->n_channels * s->n_rows_raw * n_frames;
    int blocks = (int)std::min<size_t>((total + 255) / 256, (size_t)std::max(sms, 1) * 16);
    if (blocks < 1) blocks = 1;
    phantom_project_kernel<<<blocks, 256, 0, stream>>>(d_scan, d_tube_angles, d_table_positions,
                                                      (size_t)mr->rp.n_readings, frame0, n_frames,
                                                      d_out);
    SYNTH_CUDA_TRY(cudaGetLastError());
    SYNTH_CUDA_TRY(cudaFreeAsync(d_scan, stream));
    SYNTH_CUDA_TRY(cudaStreamSynchronize(stream));
    return 0;
}

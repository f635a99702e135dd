// pmgb_api.cu -- the extern "C" boundary of libpmgb (declared in include/pmgb.h).
//
// Host-side preparation of a system: wrap and species-sort the replicated framework
// into fixed-point int4 segments, merge framework charges onto LJ sites that share their
// coordinates, merge guest LJ sites and charges, build per (segment, site) LJ
// parameters, group Ewald k-vectors into kc half-rows; then launches and status checks.
#include "pmgb.h"
#include "pmgb_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <atomic>
#include <new>
#include <string>
#include <thread>
#include <vector>

namespace {

thread_local std::string g_create_error;

constexpr double kPi = 3.14159265358979323846;
constexpr int64_t kLatencyConfs = 64;  // pmgb_energies: up to this many, one CTA per configuration

// 1/(4 pi eps0) with eps0 in e^2/(A K), following src/electrostatics.jl:6-7.
double coulomb_constant() {
    const double qe = 1.602176565e-19;
    const double eps0 = 8.854187817e-12 / (qe * qe) / 1.0e10 * 1.3806488e-23;
    return 1.0 / (4.0 * kPi * eps0);
}

struct DevBuf {
    void* p = nullptr;
    size_t n = 0;
};

}  // namespace

struct pmgb_ctx {
    int refs = 1;                   // the handle itself + one per live system or batch
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    unsigned int* d_status = nullptr;
    // device memory of systems and batches: a stream-ordered pool that keeps freed memory for
    // reuse (repeated set-up, as in a screening loop over the drop-in, allocates from the cache)
    cudaMemPool_t pool = nullptr;
    // the last erfc(alpha r)/r table built (set-up of many systems with one Ewald precision and
    // cutoff reuses it)
    double es_alpha = 0.0, es_smax = 0.0;
    std::vector<double> es_table;
    // device copies of the erfc(alpha r)/r tables built (FP64 and double-float), one per
    // (alpha, cutoff); shared by the context's systems and freed with the context
    struct EsTable {
        double alpha, smax;
        double* d_es;
        float2* d_es_df;
        int n;
    };
    std::vector<EsTable> es_tables;
    // pinned staging of host-to-device uploads: a bump region, reused from its start once the
    // stream has drained
    char* stage = nullptr;
    size_t stage_cap = 0, stage_used = 0;
    // pinned landing buffer of the structure factors read back by the unit-cell set-up (grow-only;
    // every call synchronises before it returns, so the next may reuse it)
    double* sk_host = nullptr;
    size_t sk_host_cap = 0;
    // optional CUDA events around the Widom passes' pair-kernel launches (pmgb_set_kernel_timing)
    bool timing = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> timing_events;
    size_t timing_used = 0;
    std::string err;
};

struct pmgb_system {
    pmgb_ctx* ctx = nullptr;
    int refs = 1;                   // the handle itself + one per move handle or batch holding it
    SysDev dev{};
    // device allocations
    int4* d_rec = nullptr;
    ChunkBox* d_cbox = nullptr;
    double* d_rec_q = nullptr;
    double2* d_segpar64 = nullptr;
    SegDesc* d_seg = nullptr;
    SitePar* d_segpar = nullptr;
    double* d_qxf = nullptr;         // framework charge fractional coordinates (S(k))
    double* d_rec_xf = nullptr;
    double* d_q = nullptr;
    int n_q = 0;
    KRow* d_krow = nullptr;
    float2* d_skw = nullptr;
    double* d_sk = nullptr;
    int* d_kabc = nullptr;          // k-vectors in half-row traversal order
    double* d_wt = nullptr;
    float4* d_rec_rq = nullptr;     // double-float record data of the refinement
    float* d_rec_qlo = nullptr;
    float4* d_segpar_df = nullptr;
    float4* d_tk_df = nullptr;       // wt S(k) of the evaluated k-vectors, double-float
    std::vector<int> k_order;       // traversal position -> caller's k index
    std::vector<double> h_sk;       // S(k) of every caller k-vector (re, im), caller order
    int n_k = 0;
    bool ewald_set = false;
    int n_sites = 0;
    int64_t h2d_bytes = 0;
    // host copies for the adjoint's species-pair assembly
    int n_species = 0;
    std::vector<double> eps, sig2;
    std::vector<int> seg_species;   // framework species of each segment (-1: charge-only)
    std::vector<int> site_species;  // guest LJ species of each site (-1: charge-only site)
    int site_atom[PMGB_MAX_SITES];
    int site_charge[PMGB_MAX_SITES];
    double refine_tail = 0.0;       // FP64 refinement of the Boltzmann tail (0: off)
    bool cull = true;               // spatially ordered processing with cutoff culling
    bool centre_image = true;       // centre-image distances where the geometry allows them
    int image_lists = 1;            // ordered Widom passes: image lists (csrc/pmgb_img.cu): 0 off, 1 auto, 2 on
    bool exact = true;              // single-configuration energies and grids to the FP64 tolerance
    double bound_kappa = 1.0;       // rounding condition of the box (scales the FP32 error estimate)
    DevBuf o_counts, o_perm;        // Widom processing order scratch
    DevBuf acc;                     // accessibility grid (uint8, i fastest)
    int last_refined_slot = -1;     // r_offsets entry holding the last double-float pass's count (-1: none)
    // grow-only scratch used by launches
    DevBuf r_hist, r_cut, r_counts, r_offsets, r_list, r_ref, r_plan, r_done, r_part;  // refinement scratch
    DevBuf partials, block_out, in_buf, out_buf, axes, axes64;
    DevBuf g_u, g_dsum, g_grad, g_part, g_cols;  // adjoint scratch
    DevBuf x64, e_bound;            // exact energies: FP64 site coordinates, grid error estimates
    DevBuf stats;                   // work counts of the diagnostic passes
};

namespace {

int fail(pmgb_ctx* ctx, int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (ctx) ctx->err = buf;
    else g_create_error = buf;
    return code;
}

int cuda_fail(pmgb_ctx* ctx, cudaError_t e, const char* what) {
    const int code = (e == cudaErrorMemoryAllocation) ? PMGB_ERR_OUT_OF_MEMORY : PMGB_ERR_CUDA;
    return fail(ctx, code, "%s: %s", what, cudaGetErrorString(e));
}

#define PMGB_CK(ctx, call)                                        \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return cuda_fail((ctx), e_, #call); \
    } while (0)

// Entry of every call that works on the device: select the context's device and discard an error
// left in the thread's CUDA error state by earlier, unrelated runtime calls (another library's, or
// a teardown's), so that the launch checks below report only this call's own errors.  A sticky
// error of a broken context is not hidden by this: every later call on the device returns it.
static cudaError_t enter_device(int device) {
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) (void)cudaGetLastError();
    return e;
}

// Device memory from the context's pool, ordered on its current stream (all of a context's
// work runs on that stream; pmgb_set_stream waits for the previous one).
cudaError_t dev_malloc(pmgb_ctx* ctx, void** p, size_t bytes) {
    return cudaMallocFromPoolAsync(p, bytes, ctx->pool, ctx->stream);
}
void dev_free(pmgb_ctx* ctx, void* p) {
    if (p) cudaFreeAsync(p, ctx->stream);
}

// The Widom passes' pair-kernel launch, between two CUDA events on the launching stream when
// kernel timing is on (at most 4096 launches are timed between two reads).
cudaError_t launch_pairs_timed(pmgb_ctx* ctx, const LaunchArgs& a, int n_ctas, bool img = false) {
    auto launch = [&]() {
        return img ? pmgb_launch_pairs_img(a, n_ctas, ctx->stream) : pmgb_launch_pairs(a, n_ctas, ctx->stream);
    };
    if (!ctx->timing || ctx->timing_used >= 4096) return launch();
    if (ctx->timing_used == ctx->timing_events.size()) {
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        cudaError_t e = cudaEventCreate(&e0);
        if (e == cudaSuccess) e = cudaEventCreate(&e1);
        if (e != cudaSuccess) {
            if (e0) cudaEventDestroy(e0);
            return e;
        }
        ctx->timing_events.emplace_back(e0, e1);
    }
    const auto& ev = ctx->timing_events[ctx->timing_used++];
    cudaError_t e = cudaEventRecord(ev.first, ctx->stream);
    if (e == cudaSuccess) e = launch();
    if (e == cudaSuccess) e = cudaEventRecord(ev.second, ctx->stream);
    return e;
}

int ensure(pmgb_ctx* ctx, DevBuf& b, size_t bytes) {
    if (bytes <= b.n) return PMGB_OK;
    dev_free(ctx, b.p);
    b.p = nullptr;
    b.n = 0;
    const size_t want = std::max<size_t>(bytes, 256);
    PMGB_CK(ctx, dev_malloc(ctx, &b.p, want));
    b.n = want;
    return PMGB_OK;
}

// Host-to-device copy through the context's pinned staging region: the bytes are copied there on
// the host and the transfer is enqueued without waiting for the stream (a copy from pageable
// memory would first wait for all earlier work on it), so `src` may be released on return.  When
// the region is full the stream is drained and the region reused from its start; arrays larger
// than its largest size go as plain copies.
int staged_h2d(pmgb_ctx* ctx, void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return PMGB_OK;
    constexpr size_t kMin = size_t{4} << 20, kMax = size_t{64} << 20;
    if (bytes > kMax) {
        PMGB_CK(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
        return PMGB_OK;
    }
    const size_t need = (bytes + 255) & ~size_t{255};
    if (ctx->stage_used + need > ctx->stage_cap) {
        PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));  // every staged copy has landed
        ctx->stage_used = 0;
        if (need > ctx->stage_cap) {
            if (ctx->stage) cudaFreeHost(ctx->stage);
            ctx->stage = nullptr;
            ctx->stage_cap = 0;
            size_t cap = kMin;
            while (cap < need) cap <<= 1;
            PMGB_CK(ctx, cudaMallocHost(reinterpret_cast<void**>(&ctx->stage), cap));
            ctx->stage_cap = cap;
        }
    }
    char* at = ctx->stage + ctx->stage_used;
    std::memcpy(at, src, bytes);
    PMGB_CK(ctx, cudaMemcpyAsync(dst, at, bytes, cudaMemcpyHostToDevice, ctx->stream));
    ctx->stage_used += need;
    return PMGB_OK;
}

template <class T>
int upload(pmgb_ctx* ctx, T** dst, const std::vector<T>& v, int64_t* counter = nullptr) {
    *dst = nullptr;
    if (counter) *counter += static_cast<int64_t>(v.size() * sizeof(T));
    const size_t bytes = std::max<size_t>(v.size() * sizeof(T), 16);
    PMGB_CK(ctx, dev_malloc(ctx, reinterpret_cast<void**>(dst), bytes));
    return staged_h2d(ctx, *dst, v.data(), v.size() * sizeof(T));
}

// fractional coordinate -> 32-bit fixed point (x * 2^32 mod 2^32), exact rounding in FP64
uint32_t to_fix(double x) {
    const double u = x - std::floor(x);
    return static_cast<uint32_t>(static_cast<uint64_t>(std::llround(u * 4294967296.0)) & 0xffffffffull);
}

// Read back and clear the device status word; synchronises the stream.
int check_status(pmgb_ctx* ctx) {
    unsigned int st = 0;
    PMGB_CK(ctx, cudaMemcpyAsync(&st, ctx->d_status, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (st != 0) {
        PMGB_CK(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof(unsigned int), ctx->stream));
        PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
        return fail(ctx, PMGB_ERR_DEVICE_STATUS, "kernel reported status 0x%x (%s)", st,
                    (st & PMGB_DEVERR_TMA_TIMEOUT) ? "shared-memory staging wait gave up" : "bad arguments");
    }
    return PMGB_OK;
}

bool finite3(const double* p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

double wrap01(double x) {
    double y = x - std::floor(x);
    if (y >= 1.0) y = 0.0;  // x - floor(x) can round up to 1 for tiny negative x
    return y;
}

// 3x3 helpers on column-major matrices
void inv_upper(const double R[9], double out[9]) {
    // R upper-triangular: R(i,j) = R[i + 3j], zero below the diagonal
    for (int k = 0; k < 9; ++k) out[k] = 0.0;
    const double a = R[0], b = R[3], c = R[6], d = R[4], e = R[7], f = R[8];
    out[0] = 1.0 / a;
    out[4] = 1.0 / d;
    out[8] = 1.0 / f;
    out[3] = -b / (a * d);
    out[7] = -e / (d * f);
    out[6] = (b * e - c * d) / (a * d * f);
}

// Upper-triangular R with R^T R = H^T H (Cholesky of the metric) and Q = H R^-1, so that
// |H d| = |R d| for every fractional d; Q^T maps Cartesian offsets into R's frame.
bool upper_factor(const double H[9], double R[9], double Q[9]) {
    double G[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            G[i + 3 * j] = H[3 * i] * H[3 * j] + H[3 * i + 1] * H[3 * j + 1] + H[3 * i + 2] * H[3 * j + 2];
    for (int k = 0; k < 9; ++k) R[k] = 0.0;
    if (G[0] <= 0.0) return false;
    R[0] = std::sqrt(G[0]);
    R[3] = G[3] / R[0];
    R[6] = G[6] / R[0];
    const double d11 = G[4] - R[3] * R[3];
    if (d11 <= 0.0) return false;
    R[4] = std::sqrt(d11);
    R[7] = (G[7] - R[3] * R[6]) / R[4];
    const double d22 = G[8] - R[6] * R[6] - R[7] * R[7];
    if (d22 <= 0.0) return false;
    R[8] = std::sqrt(d22);
    double Ri[9];
    inv_upper(R, Ri);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            Q[i + 3 * j] = H[i] * Ri[3 * j] + H[i + 3] * Ri[3 * j + 1] + H[i + 6] * Ri[3 * j + 2];
    return true;
}

// x as a double-float (hi, lo): hi = x rounded to FP32, lo = the FP32 remainder
inline float2 to_df(double x) {
    const float hi = static_cast<float>(x);
    return make_float2(hi, static_cast<float>(x - static_cast<double>(hi)));
}

// hash of an exact position (the bit patterns of three doubles in [0, 1))
inline size_t pos_hash(double x, double y, double z) {
    uint64_t a, b, c;
    std::memcpy(&a, &x, 8);
    std::memcpy(&b, &y, 8);
    std::memcpy(&c, &z, 8);
    uint64_t h = a * 0x9E3779B97F4A7C15ull;
    h ^= (b + 0x632BE59BD9B4E019ull) * 0xC2B2AE3D27D4EB4Full;
    h ^= h >> 29;
    h += c * 0x165667B19E3779F9ull;
    h ^= h >> 32;
    return static_cast<size_t>(h);
}

// the low 10 bits of v moved to every third bit (bit i -> bit 3 i), for Z-order codes
inline uint32_t spread10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

}  // namespace

// ============================================================================
// library / context
// ============================================================================
// the failure message of a context, for entry points defined in other translation units
int pmgb_fail_message(pmgb_ctx* ctx, int code, const char* message) { return fail(ctx, code, "%s", message); }

extern "C" int pmgb_abi_version(void) { return PMGB_ABI_VERSION; }

extern "C" int pmgb_create(int device, pmgb_ctx** out) {
    if (!out) return fail(nullptr, PMGB_ERR_INVALID_ARGUMENT, "pmgb_create: out is NULL");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return fail(nullptr, PMGB_ERR_CUDA, "pmgb_create: no CUDA device (%s)", cudaGetErrorString(e));
    if (device < 0 || device >= n)
        return fail(nullptr, PMGB_ERR_INVALID_ARGUMENT, "pmgb_create: device %d out of range [0, %d)", device, n);
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(nullptr, PMGB_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, device);
    if (prop.major < 10)
        return fail(nullptr, PMGB_ERR_UNSUPPORTED, "pmgb_create: device %d is sm_%d%d; libpmgb targets sm_103a",
                    device, prop.major, prop.minor);
    pmgb_ctx* c = new pmgb_ctx();
    c->device = device;
    e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_status, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, sizeof(unsigned int));
    if (e == cudaSuccess) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        e = cudaMemPoolCreate(&c->pool, &props);
        uint64_t keep = UINT64_MAX;  // never trim: freed blocks stay cached until the context goes
        if (e == cudaSuccess) e = cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e == cudaSuccess) e = pmgb_launch_phase_table(c->own_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->own_stream);
    if (e != cudaSuccess) {
        if (c->pool) cudaMemPoolDestroy(c->pool);
        if (c->d_status) cudaFree(c->d_status);
        if (c->own_stream) cudaStreamDestroy(c->own_stream);
        delete c;
        return fail(nullptr, PMGB_ERR_CUDA, "pmgb_create: %s", cudaGetErrorString(e));
    }
    c->stream = c->own_stream;
    *out = c;
    return PMGB_OK;
}

// Systems and batches hold a reference to their context, so handles may be destroyed in any
// order (garbage-collected hosts finalise in no particular order); the context is freed with
// its last holder.
static void ctx_release(pmgb_ctx* ctx) {
    if (--ctx->refs > 0) return;
    cudaSetDevice(ctx->device);
    if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
    cudaStreamSynchronize(ctx->stream);  // frees queued on a caller's stream
    for (auto& ev : ctx->timing_events) {
        cudaEventDestroy(ev.first);
        cudaEventDestroy(ev.second);
    }
    for (const auto& t : ctx->es_tables) {
        cudaFreeAsync(t.d_es, ctx->stream);
        cudaFreeAsync(t.d_es_df, ctx->stream);
    }
    cudaStreamSynchronize(ctx->stream);
    if (ctx->stage) cudaFreeHost(ctx->stage);
    if (ctx->sk_host) cudaFreeHost(ctx->sk_host);
    if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
    if (ctx->d_status) cudaFree(ctx->d_status);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

extern "C" void pmgb_destroy(pmgb_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->stream = ctx->own_stream;  // a caller's stream may not outlive this handle
    ctx_release(ctx);
    (void)cudaGetLastError();
}

extern "C" const char* pmgb_last_error(const pmgb_ctx* ctx) {
    return ctx ? ctx->err.c_str() : g_create_error.c_str();
}

extern "C" int pmgb_set_stream(pmgb_ctx* ctx, void* stream) {
    if (!ctx) return PMGB_ERR_INVALID_ARGUMENT;
    PMGB_CK(ctx, enter_device(ctx->device));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));  // pool memory is ordered on one stream
    ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    return PMGB_OK;
}

extern "C" int pmgb_set_kernel_timing(pmgb_ctx* ctx, int32_t on) {
    if (!ctx) return PMGB_ERR_INVALID_ARGUMENT;
    PMGB_CK(ctx, enter_device(ctx->device));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->timing = on != 0;
    ctx->timing_used = 0;
    return PMGB_OK;
}

extern "C" int pmgb_kernel_timing(pmgb_ctx* ctx, double* total_ms, int64_t* launches) {
    if (!ctx || !total_ms || !launches) return PMGB_ERR_INVALID_ARGUMENT;
    PMGB_CK(ctx, enter_device(ctx->device));
    double sum = 0.0;
    for (size_t i = 0; i < ctx->timing_used; ++i) {
        PMGB_CK(ctx, cudaEventSynchronize(ctx->timing_events[i].second));
        float ms = 0.0f;
        PMGB_CK(ctx, cudaEventElapsedTime(&ms, ctx->timing_events[i].first, ctx->timing_events[i].second));
        sum += ms;
    }
    *total_ms = sum;
    *launches = static_cast<int64_t>(ctx->timing_used);
    ctx->timing_used = 0;
    return PMGB_OK;
}

extern "C" int pmgb_synchronize(pmgb_ctx* ctx) {
    if (!ctx) return PMGB_ERR_INVALID_ARGUMENT;
    PMGB_CK(ctx, enter_device(ctx->device));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return PMGB_OK;
}

extern "C" int pmgb_test_bounded_wait(pmgb_ctx* ctx, int64_t limit_ns, int32_t arm) {
    if (!ctx) return PMGB_ERR_INVALID_ARGUMENT;
    if (limit_ns < 1 || limit_ns > 100000000)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_test_bounded_wait: limit_ns in [1, 1e8]");
    PMGB_CK(ctx, enter_device(ctx->device));
    PMGB_CK(ctx, pmgb_launch_bounded_wait_test(ctx->d_status, static_cast<unsigned long long>(limit_ns), arm ? 1 : 0,
                                               ctx->stream));
    return check_status(ctx);
}

extern "C" int pmgb_device_status(pmgb_ctx* ctx, uint32_t* status_out) {
    if (!ctx || !status_out) return PMGB_ERR_INVALID_ARGUMENT;
    PMGB_CK(ctx, enter_device(ctx->device));
    unsigned int st = 0;
    PMGB_CK(ctx, cudaMemcpyAsync(&st, ctx->d_status, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream));
    PMGB_CK(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof(unsigned int), ctx->stream));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    *status_out = st;
    return PMGB_OK;
}

// ============================================================================
// system
// ============================================================================
static void free_system_device(pmgb_system* s) {
    void* ptrs[] = {s->d_rec,      s->d_rec_q,     s->d_segpar64, s->d_seg,   s->d_segpar,  s->d_qxf,    s->d_rec_xf, s->d_q,     s->d_krow,
                    s->d_skw,      s->d_sk,        s->d_kabc,    s->d_wt,     s->partials.p, s->block_out.p,
                    s->in_buf.p,   s->out_buf.p,   s->axes.p,    s->axes64.p,    s->g_u.p,    s->g_dsum.p, s->g_grad.p,
                    s->g_part.p,   s->g_cols.p,   s->r_hist.p,  s->r_cut.p,  s->r_counts.p, s->r_offsets.p,
                    s->r_list.p,   s->r_ref.p,    s->o_counts.p, s->o_perm.p,  s->r_plan.p,  s->r_done.p,
                    s->r_part.p,   s->acc.p,      s->d_cbox,    s->d_rec_rq,
                    s->d_rec_qlo,  s->d_segpar_df, s->d_tk_df, s->x64.p,  s->e_bound.p, s->stats.p};
    for (void* p : ptrs) dev_free(s->ctx, p);
}

// Where the kernels may take every guest site's minimum image from the pose centre's (see
// run_unit): every perpendicular width W_d = 1 / |row d of c_to_f| at least 2 (rc + reach) + 0.1 A
// (rc: the larger cutoff; reach: the largest site distance from the centre).  Called whenever a
// cutoff changes.
static void set_centre_image(SysDev& D) {
    D.com_axis = -2;
    const double rc = std::sqrt(std::max(D.rc2_64, D.charged ? D.rc2e_64 : 0.0));
    const double reach = D.com_reach;
    D.com_reach2 = static_cast<float>((rc + reach) * (rc + reach) * (1.0 + 1e-6));
    if (D.n_sites < 2 || reach <= 0.0) return;
    for (int d = 0; d < 3; ++d) {
        // rows of the upper-triangular c_to_f (00 01 02 11 12 22)
        const double r0 = d == 0 ? D.g64[0] : 0.0, r1 = d == 0 ? D.g64[1] : (d == 1 ? D.g64[3] : 0.0);
        const double r2 = d == 0 ? D.g64[2] : (d == 1 ? D.g64[4] : D.g64[5]);
        if (1.0 / std::sqrt(r0 * r0 + r1 * r1 + r2 * r2) < 2.0 * (rc + reach) + 0.1) return;
    }
    D.com_axis = -1;
}

static void update_centre_image(pmgb_system* s) {
    set_centre_image(s->dev);
    if (!s->centre_image) s->dev.com_axis = -2;
}

namespace {

// Error of a step that may run off the calling thread: the code and message are kept here and
// reported through the context afterwards.
struct Err {
    int code = PMGB_OK;
    std::string msg;
    int set(int c, const char* fmt, ...) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        code = c;
        msg = buf;
        return c;
    }
};

// The arrays of pmgb_system_create.
struct CreateIn {
    const double* f_to_c;
    int32_t n_atoms;
    const double* atom_xf;
    const int32_t* atom_species;
    int32_t n_charges;
    const double* charge_xf;
    const double* charge_q;
    int32_t n_species;
    const double* epsilon;
    const double* sigma2;
    double r2_cutoff;
    int32_t n_guest_atoms;
    const double* guest_atom_x;
    const int32_t* guest_atom_species;
    int32_t n_guest_charges;
    const double* guest_charge_x;
    const double* guest_charge_q;
};

// What a system's device arrays are built from, computed on the host.
struct SysHost {
    std::vector<int4> rec;
    std::vector<double> rec_q, rec_xf;
    std::vector<float4> rec_rq;
    std::vector<float> rec_qlo;
    std::vector<SegDesc> seg;
    std::vector<SitePar> par;
    std::vector<double2> par64;
    std::vector<float4> par_df;
    std::vector<ChunkBox> cbox;
    std::vector<double> qxf, q;
    bool keep_cbox = false;  // the sub-chunk boxes are worth testing (see the estimate below)
};

}  // namespace

// Host half of pmgb_system_create: validates the arrays and fills every host-side field of s and
// the arrays of h; touches neither the device nor the context, so systems can be built on several
// threads at once.
static int system_build_host(const CreateIn& in, pmgb_system* s, SysHost& h, Err& er) {
    const double* f_to_c = in.f_to_c;
    const int32_t n_atoms = in.n_atoms, n_charges = in.n_charges, n_species = in.n_species;
    const double *atom_xf = in.atom_xf, *charge_xf = in.charge_xf, *charge_q = in.charge_q;
    const int32_t* atom_species = in.atom_species;
    const double *epsilon = in.epsilon, *sigma2 = in.sigma2;
    const double r2_cutoff = in.r2_cutoff;
    const int32_t n_guest_atoms = in.n_guest_atoms, n_guest_charges = in.n_guest_charges;
    const double *guest_atom_x = in.guest_atom_x, *guest_charge_x = in.guest_charge_x,
                 *guest_charge_q = in.guest_charge_q;
    const int32_t* guest_atom_species = in.guest_atom_species;

    if (!f_to_c) return er.set(PMGB_ERR_INVALID_ARGUMENT, "pmgb_system_create: f_to_c is NULL");
    for (int k = 0; k < 9; ++k)
        if (!std::isfinite(f_to_c[k])) return er.set(PMGB_ERR_INVALID_ARGUMENT, "f_to_c has a non-finite entry");
    if (n_atoms < 0 || n_charges < 0 || n_guest_atoms < 0 || n_guest_charges < 0 || n_species < 0)
        return er.set(PMGB_ERR_INVALID_ARGUMENT, "negative count");
    if ((n_atoms > 0 && (!atom_xf || !atom_species)) || (n_charges > 0 && (!charge_xf || !charge_q)) ||
        (n_guest_atoms > 0 && (!guest_atom_x || !guest_atom_species)) ||
        (n_guest_charges > 0 && (!guest_charge_x || !guest_charge_q)) ||
        (n_species > 0 && (!epsilon || !sigma2)))
        return er.set(PMGB_ERR_INVALID_ARGUMENT, "NULL array with a nonzero count");
    if (!(r2_cutoff > 0.0) || !std::isfinite(r2_cutoff))
        return er.set(PMGB_ERR_INVALID_ARGUMENT, "r2_cutoff must be positive and finite (got %g)", r2_cutoff);
    if (n_guest_atoms + n_guest_charges == 0)
        return er.set(PMGB_ERR_INVALID_ARGUMENT, "guest has no atoms and no charges");
    for (int i = 0; i < n_atoms; ++i) {
        if (atom_species[i] < 0 || atom_species[i] >= n_species)
            return er.set(PMGB_ERR_INVALID_ARGUMENT, "framework atom %d: species id %d not in [0, %d)", i,
                        atom_species[i], n_species);
        if (!finite3(atom_xf + 3 * i))
            return er.set(PMGB_ERR_INVALID_ARGUMENT, "framework atom %d has a non-finite coordinate", i);
    }
    for (int i = 0; i < n_charges; ++i)
        if (!finite3(charge_xf + 3 * i) || !std::isfinite(charge_q[i]))
            return er.set(PMGB_ERR_INVALID_ARGUMENT, "framework charge %d is not finite", i);
    for (int i = 0; i < n_guest_atoms; ++i) {
        if (guest_atom_species[i] < 0 || guest_atom_species[i] >= n_species)
            return er.set(PMGB_ERR_INVALID_ARGUMENT, "guest atom %d: species id %d not in [0, %d)", i,
                        guest_atom_species[i], n_species);
        if (!finite3(guest_atom_x + 3 * i))
            return er.set(PMGB_ERR_INVALID_ARGUMENT, "guest atom %d has a non-finite coordinate", i);
    }
    for (int i = 0; i < n_guest_charges; ++i)
        if (!finite3(guest_charge_x + 3 * i) || !std::isfinite(guest_charge_q[i]))
            return er.set(PMGB_ERR_INVALID_ARGUMENT, "guest charge %d is not finite", i);
    for (int k = 0; k < n_species * n_species; ++k)
        if (!std::isfinite(epsilon[k]) || !std::isfinite(sigma2[k]))
            return er.set(PMGB_ERR_INVALID_ARGUMENT, "force-field table entry %d is not finite", k);

    // ---- box: upper-triangular factor --------------------------------------------
    double R[9], Q[9], G[9];
    const double scale = std::max({std::fabs(f_to_c[0]), std::fabs(f_to_c[4]), std::fabs(f_to_c[8])});
    const bool upper = std::fabs(f_to_c[1]) <= 1e-12 * scale && std::fabs(f_to_c[2]) <= 1e-12 * scale &&
                       std::fabs(f_to_c[5]) <= 1e-12 * scale && f_to_c[0] > 0 && f_to_c[4] > 0 && f_to_c[8] > 0;
    if (upper) {
        for (int k = 0; k < 9; ++k) R[k] = f_to_c[k];
        R[1] = R[2] = R[5] = 0.0;
        for (int k = 0; k < 9; ++k) Q[k] = (k % 4 == 0) ? 1.0 : 0.0;
    } else if (!upper_factor(f_to_c, R, Q)) {
        return er.set(PMGB_ERR_INVALID_ARGUMENT, "f_to_c is singular");
    }
    inv_upper(R, G);

    // ---- framework records ---------------------------------------------------------
    struct Rec {
        double x, y, z, q;
        int species;  // -1: charge-only
    };
    std::vector<Rec> recs;  // (the local layout of a record while the segments are built)
    recs.reserve(n_atoms + n_charges);
    for (int i = 0; i < n_atoms; ++i)
        recs.push_back(Rec{wrap01(atom_xf[3 * i]), wrap01(atom_xf[3 * i + 1]), wrap01(atom_xf[3 * i + 2]), 0.0,
                           atom_species[i]});
    // a charge at exactly an atom's position merges into the first such atom, unless an earlier
    // charge took it: an open-addressing table from exact positions to the first atom there
    size_t cap = 16;
    while (cap < 2 * static_cast<size_t>(n_atoms)) cap <<= 1;
    std::vector<int> slot(cap, -1);
    auto probe = [&](double x, double y, double z) {
        size_t h = pos_hash(x, y, z) & (cap - 1);
        while (slot[h] >= 0) {
            const Rec& o = recs[slot[h]];
            if (o.x == x && o.y == y && o.z == z) break;
            h = (h + 1) & (cap - 1);
        }
        return h;
    };
    for (int i = 0; i < n_atoms; ++i) {
        const size_t h = probe(recs[i].x, recs[i].y, recs[i].z);
        if (slot[h] < 0) slot[h] = i;
    }
    std::vector<char> taken(recs.size(), 0);
    for (int c = 0; c < n_charges; ++c) {
        const double x = wrap01(charge_xf[3 * c]), y = wrap01(charge_xf[3 * c + 1]), z = wrap01(charge_xf[3 * c + 2]);
        const int hit = n_atoms > 0 ? slot[probe(x, y, z)] : -1;
        if (hit >= 0 && !taken[hit]) {
            recs[hit].q = charge_q[c];
            taken[hit] = 1;
        } else {
            recs.push_back(Rec{x, y, z, charge_q[c], -1});
        }
    }
    // species-sorted contiguous segments of fixed-point records; within a segment, Z-order of the
    // position (10 bits per axis): consecutive records are spatially close, so a warp can skip
    // groups of them that lie beyond the cutoff.  Sort keys (species, Z code, index) packed in 64
    // bits: 7 + 30 + 27 (index last, so equal codes keep their input order).
    if (recs.size() >= (size_t{1} << 27))
        return er.set(PMGB_ERR_UNSUPPORTED, "framework has %zu records (max 2^27)", recs.size());
    std::vector<uint64_t> skey(recs.size());
    for (size_t i = 0; i < recs.size(); ++i) {
        const uint32_t zc = spread10(to_fix(recs[i].x) >> 22) | spread10(to_fix(recs[i].y) >> 22) << 1 |
                            spread10(to_fix(recs[i].z) >> 22) << 2;
        const uint64_t sp = static_cast<uint64_t>(recs[i].species < 0 ? n_species : recs[i].species);
        skey[i] = (sp << 57) | (static_cast<uint64_t>(zc) << 27) | i;
    }
    std::sort(skey.begin(), skey.end());
    std::vector<int> order(recs.size());
    for (size_t i = 0; i < recs.size(); ++i) order[i] = static_cast<int>(skey[i] & ((uint64_t{1} << 27) - 1));
    std::vector<int4>& h_rec = h.rec;
    std::vector<double>& h_rec_q = h.rec_q;      // FP64 charge of each record
    std::vector<double>& h_rec_xf = h.rec_xf;    // its exact fractional coordinates
    std::vector<float4>& h_rec_rq = h.rec_rq;    // position beyond the fixed point (units of 2^-32), q hi
    std::vector<float>& h_rec_qlo = h.rec_qlo;   // q lo
    std::vector<SegDesc>& h_seg = h.seg;
    for (size_t p = 0; p < order.size();) {
        const int sp = recs[order[p]].species;
        size_t e = p;
        while (e < order.size() && recs[order[e]].species == sp) ++e;
        SegDesc d{};
        d.lo = static_cast<int>(h_rec.size());
        for (size_t k = p; k < e; ++k) {
            const Rec& r = recs[order[k]];
            const float qf = static_cast<float>(r.q);
            int qbits;
            std::memcpy(&qbits, &qf, sizeof(qbits));
            h_rec.push_back(make_int4(static_cast<int>(to_fix(r.x)), static_cast<int>(to_fix(r.y)),
                                      static_cast<int>(to_fix(r.z)), qbits));
            h_rec_q.push_back(r.q);
            h_rec_xf.push_back(r.x);
            h_rec_xf.push_back(r.y);
            h_rec_xf.push_back(r.z);
            // the fixed point rounds u 2^32 to the nearest integer (mod 2^32): keep the remainder
            const double rx = r.x * 4294967296.0 - static_cast<double>(std::llround(r.x * 4294967296.0));
            const double ry = r.y * 4294967296.0 - static_cast<double>(std::llround(r.y * 4294967296.0));
            const double rz = r.z * 4294967296.0 - static_cast<double>(std::llround(r.z * 4294967296.0));
            const float2 qd = to_df(r.q);
            h_rec_rq.push_back(make_float4(static_cast<float>(rx), static_cast<float>(ry), static_cast<float>(rz), qd.x));
            h_rec_qlo.push_back(qd.y);
        }
        d.hi = static_cast<int>(h_rec.size());
        d.species = sp;
        d.has_lj = sp >= 0;
        h_seg.push_back(d);
        p = e;
    }
    if (h_seg.size() > PMGB_MAX_SEG)
        return er.set(PMGB_ERR_UNSUPPORTED, "framework has %zu species segments (max %d)", h_seg.size(),
                    PMGB_MAX_SEG);

    // ---- guest sites: merge LJ atoms and charges sharing an offset -------------------
    double body[PMGB_MAX_SITES][3];
    double sq[PMGB_MAX_SITES];
    int ns = 0;
    for (int i = 0; i < n_guest_atoms; ++i) {
        if (ns >= PMGB_MAX_SITES) return er.set(PMGB_ERR_UNSUPPORTED, "guest has more than %d sites", PMGB_MAX_SITES);
        for (int d = 0; d < 3; ++d) body[ns][d] = guest_atom_x[3 * i + d];
        s->site_atom[ns] = i;
        s->site_charge[ns] = -1;
        sq[ns] = 0.0;
        ++ns;
    }
    for (int c = 0; c < n_guest_charges; ++c) {
        int hit = -1;
        for (int k = 0; k < ns; ++k) {
            if (s->site_charge[k] >= 0) continue;
            const double dd = std::fabs(body[k][0] - guest_charge_x[3 * c]) +
                              std::fabs(body[k][1] - guest_charge_x[3 * c + 1]) +
                              std::fabs(body[k][2] - guest_charge_x[3 * c + 2]);
            if (dd <= 1e-12) {
                hit = k;
                break;
            }
        }
        if (hit < 0) {
            if (ns >= PMGB_MAX_SITES)
                return er.set(PMGB_ERR_UNSUPPORTED, "guest has more than %d sites", PMGB_MAX_SITES);
            hit = ns++;
            for (int d = 0; d < 3; ++d) body[hit][d] = guest_charge_x[3 * c + d];
            s->site_atom[hit] = -1;
        }
        s->site_charge[hit] = c;
        sq[hit] = guest_charge_q[c];
    }
    s->n_sites = ns;
    s->n_species = n_species;
    s->eps.assign(epsilon, epsilon + static_cast<size_t>(n_species) * n_species);
    s->sig2.assign(sigma2, sigma2 + static_cast<size_t>(n_species) * n_species);
    for (const SegDesc& d : h_seg) s->seg_species.push_back(d.species);
    for (int k = 0; k < ns; ++k) s->site_species.push_back(s->site_atom[k] >= 0 ? guest_atom_species[s->site_atom[k]] : -1);

    // per (segment, site) LJ parameters
    std::vector<SitePar>& h_par = h.par;
    std::vector<double2>& h_par64 = h.par64;
    std::vector<float4>& h_par_df = h.par_df;
    h_par.assign(h_seg.size() * PMGB_MAX_SITES, SitePar{1.0f, 0.0f, -1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f});
    h_par64.assign(h_seg.size() * PMGB_MAX_SITES, make_double2(-1.0, 0.0));  // -1: no LJ
    h_par_df.assign(h_seg.size() * PMGB_MAX_SITES, make_float4(-1.0f, 0.0f, 0.0f, 0.0f));
    for (size_t g = 0; g < h_seg.size(); ++g)
        for (int k = 0; k < ns; ++k) {
            const int a = s->site_atom[k];
            const int fs = h_seg[g].species;
            if (a < 0 || fs < 0) continue;
            const int gs = guest_atom_species[a];
            SitePar& p = h_par[g * PMGB_MAX_SITES + k];
            const double s2 = sigma2[gs * n_species + fs], e4 = 4.0 * epsilon[gs * n_species + fs];
            p.sig2 = static_cast<float>(s2);
            p.eps4 = static_cast<float>(e4);
            p.lj12 = static_cast<float>(e4 * s2 * s2 * s2 * s2 * s2 * s2);
            p.lj6 = static_cast<float>(-e4 * s2 * s2 * s2);
            p.r2ovl = 0.1f;  // R²_OVERLAP, src/vdw_energetics.jl:2
            h_par64[g * PMGB_MAX_SITES + k] = make_double2(s2, e4);
            const float2 s2d = to_df(s2), e4d = to_df(e4);
            h_par_df[g * PMGB_MAX_SITES + k] = make_float4(s2d.x, s2d.y, e4d.x, e4d.y);
        }

    // bounding box of every sub-chunk of records, in the kernels' traversal order
    std::vector<ChunkBox>& h_cbox = h.cbox;
    {
        const int n_rec = static_cast<int>(h_rec.size());
        for (int t0 = 0; t0 < n_rec; t0 += PMGB_TILE) {
            const int t1 = std::min(t0 + PMGB_TILE, n_rec);
            for (const SegDesc& d : h_seg) {
                const int lo = std::max(d.lo, t0), hi = std::min(d.hi, t1);
                for (int c0 = lo; c0 < hi; c0 += PMGB_CHUNK)
                for (int j0 = c0; j0 < std::min(c0 + PMGB_CHUNK, hi); j0 += PMGB_SUBCHUNK) {
                    const int j1 = std::min({j0 + PMGB_SUBCHUNK, c0 + PMGB_CHUNK, hi});
                    uint32_t mn[3] = {UINT32_MAX, UINT32_MAX, UINT32_MAX}, mx[3] = {0, 0, 0};
                    for (int j = j0; j < j1; ++j) {
                        const uint32_t u[3] = {static_cast<uint32_t>(h_rec[j].x), static_cast<uint32_t>(h_rec[j].y),
                                               static_cast<uint32_t>(h_rec[j].z)};
                        for (int a = 0; a < 3; ++a) {
                            mn[a] = std::min(mn[a], u[a]);
                            mx[a] = std::max(mx[a], u[a]);
                        }
                    }
                    ChunkBox b{};
                    uint32_t* c = &b.cx;
                    uint32_t* e = &b.ex;
                    for (int a = 0; a < 3; ++a) {
                        const uint32_t span = mx[a] - mn[a];
                        c[a] = mn[a] + span / 2;
                        e[a] = span - span / 2 + 1;  // every record within e of the centre
                    }
                    h_cbox.push_back(b);
                }
            }
        }
    }

    // charge fractional coordinates for S(k), FP64
    std::vector<double>& h_qxf = h.qxf;
    std::vector<double>& h_q = h.q;
    for (int c = 0; c < n_charges; ++c) {
        for (int d = 0; d < 3; ++d) h_qxf.push_back(wrap01(charge_xf[3 * c + d]));
        h_q.push_back(charge_q[c]);
    }
    s->n_q = n_charges;

    SysDev& D = s->dev;
    {
        // skipping pays only where sub-chunks often lie beyond the cutoff of a compact group of
        // sites: estimate the skipped fraction 1 - (4/3) pi (rc + rho)^3 / V per sub-chunk (rho:
        // the Cartesian radius of its box, largest over the corners) and keep the boxes only if
        // it averages at least 0.1 (the box tests cost a few per cent where nothing is skipped)
        const double vol = std::fabs(R[0] * R[4] * R[8]);
        const double rc = std::sqrt(r2_cutoff);
        double skip = 0.0;
        for (const ChunkBox& b : h_cbox) {
            const double e[3] = {b.ex / 4294967296.0, b.ey / 4294967296.0, b.ez / 4294967296.0};
            double rho2 = 0.0;
            for (int sgn = 0; sgn < 4; ++sgn) {
                const double f[3] = {e[0], (sgn & 1) ? -e[1] : e[1], (sgn & 2) ? -e[2] : e[2]};
                double v2 = 0.0;
                for (int i = 0; i < 3; ++i) {
                    const double v = R[i] * f[0] + R[i + 3] * f[1] + R[i + 6] * f[2];
                    v2 += v * v;
                }
                rho2 = std::max(rho2, v2);
            }
            const double r = rc + std::sqrt(rho2);
            skip += std::max(0.0, 1.0 - 4.0 / 3.0 * M_PI * r * r * r / vol);
        }
        h.keep_cbox = !h_cbox.empty() && skip >= 0.1 * static_cast<double>(h_cbox.size());
    }
    {
        // perpendicular width W_d = 1 / |row d of c_to_f|; unit face normals n_d = row / |row|
        double n[3][3], w[3];
        for (int d = 0; d < 3; ++d) {
            const double r0 = G[d], r1 = G[d + 3], r2 = G[d + 6];
            const double len = std::sqrt(r0 * r0 + r1 * r1 + r2 * r2);
            w[d] = 1.0 / len;
            n[d][0] = r0 / len;
            n[d][1] = r1 / len;
            n[d][2] = r2 / len;
        }
        double lam = 0.0;  // Gershgorin bound of the largest eigenvalue of (n_i . n_j)
        for (int i = 0; i < 3; ++i) {
            double row = 0.0;
            for (int j = 0; j < 3; ++j) row += std::fabs(n[i][0] * n[j][0] + n[i][1] * n[j][1] + n[i][2] * n[j][2]);
            lam = std::max(lam, row);
        }
        for (int d = 0; d < 3; ++d) D.cw[d] = static_cast<float>(w[d] / 4294967296.0 * (1.0 - 1e-6));
        D.cw_inv_lam = static_cast<float>((1.0 - 1e-6) / lam);
    }
    D.n_rec = static_cast<int>(h_rec.size());
    D.n_tiles = (D.n_rec + PMGB_TILE - 1) / PMGB_TILE;
    D.n_seg = static_cast<int>(h_seg.size());
    const double fix_unit = 1.0 / 4294967296.0;  // one fixed-point step of a fractional coordinate
    D.h00 = static_cast<float>(R[0] * fix_unit);
    D.h01 = static_cast<float>(R[3] * fix_unit);
    D.h02 = static_cast<float>(R[6] * fix_unit);
    D.h11 = static_cast<float>(R[4] * fix_unit);
    D.h12 = static_cast<float>(R[7] * fix_unit);
    D.h22 = static_cast<float>(R[8] * fix_unit);
    D.p00 = static_cast<float>(R[0] * fix_unit - static_cast<double>(D.h00));
    D.p01 = static_cast<float>(R[3] * fix_unit - static_cast<double>(D.h01));
    D.p02 = static_cast<float>(R[6] * fix_unit - static_cast<double>(D.h02));
    D.p11 = static_cast<float>(R[4] * fix_unit - static_cast<double>(D.h11));
    D.p12 = static_cast<float>(R[7] * fix_unit - static_cast<double>(D.h12));
    D.p22 = static_cast<float>(R[8] * fix_unit - static_cast<double>(D.h22));
    D.g00 = static_cast<float>(G[0]);
    D.g01 = static_cast<float>(G[3]);
    D.g02 = static_cast<float>(G[6]);
    D.g11 = static_cast<float>(G[4]);
    D.g12 = static_cast<float>(G[7]);
    D.g22 = static_cast<float>(G[8]);
    const int up[6] = {0, 3, 6, 4, 7, 8};  // column-major indices of the upper triangle
    for (int i = 0; i < 6; ++i) {
        D.f2c64[i] = R[up[i]];
        D.g64[i] = G[up[i]];
        D.h_df[i] = to_df(R[up[i]] * fix_unit);
    }
    // rounding condition of the box, || |R| |R^-1| ||_inf (1 for an orthorhombic cell): how much
    // the FP32 Cartesian conversion of a fractional displacement can amplify its roundings
    s->bound_kappa = 1.0;
    for (int i = 0; i < 3; ++i) {
        double row = 0.0;
        for (int j = 0; j < 3; ++j)
            for (int m = 0; m < 3; ++m) row += std::fabs(R[i + 3 * m]) * std::fabs(G[m + 3 * j]);
        s->bound_kappa = std::max(s->bound_kappa, row);
    }
    D.rc2_df = to_df(r2_cutoff);
    D.rc2e_df = D.rc2_df;
    D.es_tab_df = nullptr;
    D.es_n_oct = 0;
    D.rc2 = static_cast<float>(r2_cutoff);
    D.rc2e = static_cast<float>(r2_cutoff);
    D.alpha = 0.0f;
    D.rc2_64 = r2_cutoff;
    D.rc2e_64 = r2_cutoff;
    D.alpha64 = 0.0;
    D.sk64 = nullptr;
    D.wt64 = nullptr;
    D.kabc = nullptr;
    D.coul = coulomb_constant();
    D.charged = (n_charges > 0 && n_guest_charges > 0) ? 1 : 0;
    D.n_sites = ns;
    for (int k = 0; k < PMGB_MAX_SITES; ++k) {
        // offsets rotated into the frame of the upper-triangular box (Q^T b)
        for (int d = 0; d < 3; ++d) {
            double v = 0.0;
            if (k < ns)
                for (int m = 0; m < 3; ++m) v += Q[m + 3 * d] * body[k][m];
            D.body[k][d] = static_cast<float>(v);
            D.body64[k][d] = v;
        }
        D.q[k] = (k < ns) ? static_cast<float>(sq[k]) : 0.0f;
        D.q64[k] = (k < ns) ? sq[k] : 0.0;
    }
    {
        double reach = 0.0;
        for (int k = 0; k < ns; ++k)
            reach = std::max(reach, std::sqrt(D.body64[k][0] * D.body64[k][0] + D.body64[k][1] * D.body64[k][1] +
                                              D.body64[k][2] * D.body64[k][2]));
        D.com_reach = reach > 0.0 ? static_cast<float>(reach * (1.0 + 1e-6) + 1e-4) : 0.0f;
    }
    // mirror sites: the offsets are formed by sums of exactly negated products, and the poses
    // round them to fixed point by an odd function, so site 2's offset from site 0 is exactly
    // minus site 1's in every pose
    D.k_mirror = 0;
    if (ns == 3 && D.q[1] == D.q[2]) {
        bool m = true;
        for (int d = 0; d < 3; ++d) m = m && D.body64[0][d] == 0.0 && D.body64[1][d] == -D.body64[2][d];
        D.k_mirror = m ? 1 : 0;
    }
    update_centre_image(s);
    D.n_krow = 0;
    D.n_k = 0;
    D.krow = nullptr;
    D.skw = nullptr;
    D.ks[0] = D.ks[1] = D.ks[2] = 1;
    return PMGB_OK;
}

// Device half: allocate and fill the system's arrays from h (ordered on the context's stream;
// the copies are staged through pinned memory, so h may be released when this returns) and set
// the device pointers of s->dev.
static int system_upload(pmgb_ctx* ctx, pmgb_system* s, const SysHost& h) {
    int rc = PMGB_OK;
    int64_t* nb = &s->h2d_bytes;
    if ((rc = upload(ctx, &s->d_rec, h.rec, nb)) || (rc = upload(ctx, &s->d_cbox, h.cbox, nb)) ||
        (rc = upload(ctx, &s->d_rec_q, h.rec_q, nb)) || (rc = upload(ctx, &s->d_segpar64, h.par64, nb)) ||
        (rc = upload(ctx, &s->d_seg, h.seg, nb)) || (rc = upload(ctx, &s->d_segpar, h.par, nb)) ||
        (rc = upload(ctx, &s->d_qxf, h.qxf, nb)) || (rc = upload(ctx, &s->d_rec_xf, h.rec_xf, nb)) ||
        (rc = upload(ctx, &s->d_rec_rq, h.rec_rq, nb)) || (rc = upload(ctx, &s->d_rec_qlo, h.rec_qlo, nb)) ||
        (rc = upload(ctx, &s->d_segpar_df, h.par_df, nb)) || (rc = upload(ctx, &s->d_q, h.q, nb)))
        return rc;
    SysDev& D = s->dev;
    D.rec = s->d_rec;
    D.cbox = h.keep_cbox ? s->d_cbox : nullptr;
    D.seg = s->d_seg;
    D.segpar = s->d_segpar;
    D.rec_rq = s->d_rec_rq;
    D.rec_qlo = s->d_rec_qlo;
    D.segpar_df = s->d_segpar_df;
    D.rec_q = s->d_rec_q;
    D.rec_xf = s->d_rec_xf;
    D.segpar64 = s->d_segpar64;
    return PMGB_OK;
}

extern "C" int pmgb_system_create(pmgb_ctx* ctx, const double f_to_c[9], int32_t n_atoms, const double* atom_xf,
                                  const int32_t* atom_species, int32_t n_charges, const double* charge_xf,
                                  const double* charge_q, int32_t n_species, const double* epsilon,
                                  const double* sigma2, double r2_cutoff, int32_t n_guest_atoms,
                                  const double* guest_atom_x, const int32_t* guest_atom_species,
                                  int32_t n_guest_charges, const double* guest_charge_x,
                                  const double* guest_charge_q, pmgb_system** out) {
    if (!ctx) return PMGB_ERR_INVALID_ARGUMENT;
    if (!out) return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_system_create: out is NULL");
    *out = nullptr;
    const CreateIn in{f_to_c,       n_atoms,      atom_xf,       atom_species,       n_charges,
                      charge_xf,    charge_q,     n_species,     epsilon,            sigma2,
                      r2_cutoff,    n_guest_atoms, guest_atom_x, guest_atom_species, n_guest_charges,
                      guest_charge_x, guest_charge_q};
    pmgb_system* s = new pmgb_system();
    s->ctx = ctx;
    SysHost h;
    Err er;
    if (system_build_host(in, s, h, er) != PMGB_OK) {
        delete s;
        return fail(ctx, er.code, "%s", er.msg.c_str());
    }
    const cudaError_t e0 = enter_device(ctx->device);
    int rc = e0 != cudaSuccess ? cuda_fail(ctx, e0, "cudaSetDevice") : system_upload(ctx, s, h);
    if (rc == PMGB_OK) {
        const cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = cuda_fail(ctx, e, "pmgb_system_create upload");
    }
    if (rc != PMGB_OK) {
        free_system_device(s);
        delete s;
        return rc;
    }
    ++ctx->refs;
    *out = s;
    return PMGB_OK;
}

namespace {

// Piecewise polynomial of f(s) = erfc(alpha sqrt(s)) / sqrt(s) for the FP64 refinement: octaves
// of s from 2^PMGB_ES_E_LO up to the first power of two above s_max, each cut into PMGB_ES_SUB
// intervals; on each, the degree-7 Chebyshev interpolant at 8 nodes (from the C library's erfc),
// written out as monomial coefficients in t in [-1, 1].
std::vector<double> erfc_over_r_table(double alpha, double s_max) {
    int e_hi = 0;
    std::frexp(s_max, &e_hi);  // s_max < 2^e_hi
    const int n = PMGB_ES_COEF;
    // cos(j pi (k + 1/2) / n): the Chebyshev nodes (j = 1) and the T_j values at them
    static const auto cheb = [] {
        std::vector<double> c(PMGB_ES_COEF * PMGB_ES_COEF);
        for (int j = 0; j < PMGB_ES_COEF; ++j)
            for (int k = 0; k < PMGB_ES_COEF; ++k) c[j * PMGB_ES_COEF + k] = std::cos(j * M_PI * (k + 0.5) / PMGB_ES_COEF);
        return c;
    }();
    std::vector<double> tab;
    tab.reserve(static_cast<size_t>(std::max(0, e_hi - PMGB_ES_E_LO)) * PMGB_ES_SUB * n);
    for (int e = PMGB_ES_E_LO; e < e_hi; ++e)
        for (int m = 0; m < PMGB_ES_SUB; ++m) {
            const double a = std::ldexp(1.0 + static_cast<double>(m) / PMGB_ES_SUB, e);
            const double b = std::ldexp(1.0 + static_cast<double>(m + 1) / PMGB_ES_SUB, e);
            double fk[PMGB_ES_COEF], tk[PMGB_ES_COEF];
            for (int k = 0; k < n; ++k) {
                tk[k] = cheb[n + k];
                const double sv = 0.5 * (a + b) + 0.5 * (b - a) * tk[k];
                const double r = std::sqrt(sv);
                fk[k] = std::erfc(alpha * r) / r;
            }
            // Chebyshev coefficients c_j = (2/n) sum_k f_k T_j(t_k) (c_0 halved), then the sum of
            // c_j T_j in the monomial basis through T_{j+1} = 2 t T_j - T_{j-1}
            double poly[PMGB_ES_COEF] = {}, tm1[PMGB_ES_COEF] = {}, tj[PMGB_ES_COEF] = {};
            tj[0] = 1.0;
            for (int j = 0; j < n; ++j) {
                double c = 0.0;
                for (int k = 0; k < n; ++k) c += fk[k] * cheb[j * n + k];
                c *= (j == 0 ? 1.0 : 2.0) / n;
                for (int i = 0; i < n; ++i) poly[i] += c * tj[i];
                double next[PMGB_ES_COEF] = {};
                for (int i = 0; i < n; ++i) {
                    if (i + 1 < n) next[i + 1] += 2.0 * tj[i];
                    next[i] -= (j == 0) ? 0.0 : tm1[i];
                }
                if (j == 0)  // T_1 = t
                    for (int i = 0; i < n; ++i) next[i] = (i == 1) ? 1.0 : 0.0;
                std::copy(tj, tj + n, tm1);
                std::copy(next, next + n, tj);
            }
            tab.insert(tab.end(), poly, poly + n);
        }
    return tab;
}

}  // namespace

// The device erfc(alpha r)/r tables (FP64 and double-float) for (alpha, s_max = cutoff^2): built
// and uploaded on first use, then shared by every system of the context with that Ewald set-up.
static int es_table_for(pmgb_ctx* ctx, double alpha, double smax, const pmgb_ctx::EsTable** out) {
    for (const auto& t : ctx->es_tables)
        if (t.alpha == alpha && t.smax == smax) {
            *out = &t;
            return PMGB_OK;
        }
    if (ctx->es_table.empty() || ctx->es_alpha != alpha || ctx->es_smax != smax) {
        ctx->es_table = erfc_over_r_table(alpha, smax);
        ctx->es_alpha = alpha;
        ctx->es_smax = smax;
    }
    const std::vector<double>& es = ctx->es_table;
    std::vector<float2> es_df(es.size());
    for (size_t i = 0; i < es.size(); ++i) es_df[i] = to_df(es[i]);
    pmgb_ctx::EsTable t{alpha, smax, nullptr, nullptr, static_cast<int>(es.size())};
    int rc = upload(ctx, &t.d_es, es);
    if (rc == PMGB_OK) rc = upload(ctx, &t.d_es_df, es_df);
    if (rc != PMGB_OK) {
        dev_free(ctx, t.d_es);
        dev_free(ctx, t.d_es_df);
        return rc;
    }
    ctx->es_tables.push_back(t);
    *out = &ctx->es_tables.back();
    return PMGB_OK;
}

namespace {

// Ewald state of a system computed on the host before S(k) is known: the caller's k-vectors
// grouped into half-rows.
struct EwaldHost {
    double alpha = 0.0, sr_cutoff = 0.0;
    int n_kvecs = 0;
    std::vector<KRow> rows;
    std::vector<int> order;  // traversal position -> caller's k index
    std::vector<int> kabc;   // k-vectors in traversal order
    std::vector<double> wt;
    int kmax[3] = {0, 0, 0};
};

// ... and after S(k): the k-vectors kept (every one, or the multiples of the replica strides).
struct EwaldFinal {
    int ks[3] = {1, 1, 1};
    bool pruned = false;
    std::vector<KRow> rows;
    std::vector<int> kabc;
    std::vector<double> wt, sk;
    std::vector<float2> skw;
    std::vector<float4> tk;   // wt S(k) as double-float, the kept k-vectors
    std::vector<double> h_sk; // S(k) of every caller k-vector (re, im), caller order
};

// Validate the Ewald arguments and group the k-vectors: runs of constant (ka, kb) and consecutive
// kc, each split at kc = 0 into half-rows that start at the kc nearest 0 and step outward.
// Host only (thread-safe).
int ewald_build_host(double alpha, double sr_cutoff, int32_t n_kvecs, const int32_t* kvec_abc, const double* kvec_wt,
                     EwaldHost& eh, Err& er) {
    if (!(alpha > 0.0) || !std::isfinite(alpha) || !(sr_cutoff > 0.0) || !std::isfinite(sr_cutoff))
        return er.set(PMGB_ERR_INVALID_ARGUMENT, "Ewald alpha and sr_cutoff must be positive and finite");
    if (n_kvecs < 0 || (n_kvecs > 0 && (!kvec_abc || !kvec_wt)))
        return er.set(PMGB_ERR_INVALID_ARGUMENT, "bad k-vector arrays");
    for (int k = 0; k < n_kvecs; ++k)
        if (!std::isfinite(kvec_wt[k])) return er.set(PMGB_ERR_INVALID_ARGUMENT, "k-vector %d weight not finite", k);
    eh.alpha = alpha;
    eh.sr_cutoff = sr_cutoff;
    eh.n_kvecs = n_kvecs;
    for (int k = 0; k < n_kvecs;) {
        const int ka = kvec_abc[3 * k], kb = kvec_abc[3 * k + 1], lo = kvec_abc[3 * k + 2];
        int e = k + 1;
        while (e < n_kvecs && kvec_abc[3 * e] == ka && kvec_abc[3 * e + 1] == kb &&
               kvec_abc[3 * e + 2] == kvec_abc[3 * (e - 1) + 2] + 1)
            ++e;
        const int hi = lo + (e - k) - 1;
        auto add_row = [&](int kc_start, int kc_end, int dir) {
            KRow r{ka, kb, kc_start, 0, static_cast<int>(eh.order.size()), dir, 0, 0};
            for (int kc = kc_start;; kc += dir) {
                const int idx = k + (kc - lo);
                eh.order.push_back(idx);
                eh.kabc.push_back(ka);
                eh.kabc.push_back(kb);
                eh.kabc.push_back(kc);
                eh.wt.push_back(kvec_wt[idx]);
                ++r.n;
                if (kc == kc_end) break;
            }
            eh.rows.push_back(r);
        };
        if (lo >= 0) {
            add_row(lo, hi, +1);
        } else if (hi < 0) {
            add_row(hi, lo, -1);
        } else {
            add_row(0, hi, +1);
            add_row(-1, lo, -1);
        }
        k = e;
    }
    for (int i = 0; i < n_kvecs; ++i)
        for (int d = 0; d < 3; ++d) eh.kmax[d] = std::max(eh.kmax[d], std::abs(eh.kabc[3 * i + d]));
    return PMGB_OK;
}

}  // namespace

// Drop the system's previous Ewald state, upload the k-vectors and enqueue S(k) of the framework
// charges (FP64, on the device) and its copy into sk_host (2 n_kvecs doubles, traversal order).
// Asynchronous when sk_host is pinned; the caller synchronises before reading it.
static int ewald_launch_sk(pmgb_ctx* ctx, pmgb_system* s, const EwaldHost& eh, double* sk_host) {
    void* old[] = {s->d_krow, s->d_skw, s->d_sk, s->d_kabc, s->d_wt, s->d_tk_df};
    for (void* p : old) dev_free(ctx, p);
    s->d_krow = nullptr;
    s->d_skw = nullptr;
    s->d_sk = nullptr;
    s->d_kabc = nullptr;
    s->d_wt = nullptr;
    s->d_tk_df = nullptr;
    s->ewald_set = false;
    const int n_kvecs = eh.n_kvecs;
    int rc;
    if ((rc = upload(ctx, &s->d_kabc, eh.kabc, &s->h2d_bytes)) || (rc = upload(ctx, &s->d_wt, eh.wt, &s->h2d_bytes)))
        return rc;
    PMGB_CK(ctx, dev_malloc(ctx, reinterpret_cast<void**>(&s->d_skw), std::max<size_t>(sizeof(float2) * n_kvecs, 16)));
    PMGB_CK(ctx, dev_malloc(ctx, reinterpret_cast<void**>(&s->d_sk), std::max<size_t>(2 * sizeof(double) * n_kvecs, 16)));
    double2* d_table = nullptr;  // per-axis phasors of every charge, freed once S(k) is built
    const size_t table_len = pmgb_structure_factor_table_len(s->n_q, eh.kmax);
    PMGB_CK(ctx, dev_malloc(ctx, reinterpret_cast<void**>(&d_table), std::max<size_t>(sizeof(double2) * table_len, 16)));
    const cudaError_t e_sk = pmgb_launch_structure_factor(s->d_qxf, s->d_q, s->n_q, s->d_kabc, s->d_wt, n_kvecs,
                                                          eh.kmax, d_table, s->d_sk, s->d_skw, ctx->stream);
    dev_free(ctx, d_table);
    PMGB_CK(ctx, e_sk);
    if (n_kvecs > 0)
        PMGB_CK(ctx, cudaMemcpyAsync(sk_host, s->d_sk, 2 * sizeof(double) * n_kvecs, cudaMemcpyDeviceToHost,
                                     ctx->stream));
    return PMGB_OK;
}

// S(k) of a supercell of rep[0] x rep[1] x rep[2] exact copies of a unit cell, from the unit cell:
// S(k) vanishes unless rep_d | k_d for every d, and then equals n_img S_cell(k / rep) (the copies'
// phases are all 1), so only those k-vectors are evaluated, over the unit cell's charges (unit_q_xf:
// its fractional coordinates), n_img^2 times less work than the supercell sum.  Drops the system's
// previous Ewald state and enqueues the evaluation and its copy into sk_host (2 per index of
// unit_idx, the traversal positions of the multiples, which this fills).  The device arrays of the
// k-vectors are made afterwards by ewald_upload_finish.
static int ewald_launch_sk_unit(pmgb_ctx* ctx, pmgb_system* s, const EwaldHost& eh, const int32_t rep[3], int n_uq,
                                const double* unit_q_xf, const double* unit_q, std::vector<int>& unit_idx,
                                double* sk_host) {
    void* old[] = {s->d_krow, s->d_skw, s->d_sk, s->d_kabc, s->d_wt, s->d_tk_df};
    for (void* p : old) dev_free(ctx, p);
    s->d_krow = nullptr;
    s->d_skw = nullptr;
    s->d_sk = nullptr;
    s->d_kabc = nullptr;
    s->d_wt = nullptr;
    s->d_tk_df = nullptr;
    s->ewald_set = false;
    std::vector<int> kr;
    std::vector<double> wr;
    int kmax[3] = {0, 0, 0};
    unit_idx.clear();
    for (int i = 0; i < eh.n_kvecs; ++i) {
        const int* k = &eh.kabc[3 * i];
        if (k[0] % rep[0] || k[1] % rep[1] || k[2] % rep[2]) continue;
        unit_idx.push_back(i);
        for (int d = 0; d < 3; ++d) {
            kr.push_back(k[d] / rep[d]);
            kmax[d] = std::max(kmax[d], std::abs(k[d] / rep[d]));
        }
        wr.push_back(eh.wt[i]);
    }
    const int n_r = static_cast<int>(unit_idx.size());
    if (n_r == 0) return PMGB_OK;
    std::vector<double> qxf(3 * static_cast<size_t>(n_uq)), q(unit_q, unit_q + n_uq);
    for (size_t i = 0; i < qxf.size(); ++i) qxf[i] = wrap01(unit_q_xf[i]);
    int *d_k = nullptr;
    double *d_w = nullptr, *d_qxf = nullptr, *d_q = nullptr, *d_sk = nullptr;
    float2* d_skw = nullptr;
    double2* d_table = nullptr;
    const size_t table_len = pmgb_structure_factor_table_len(n_uq, kmax);
    int rc = upload(ctx, &d_k, kr);
    if (rc == PMGB_OK) rc = upload(ctx, &d_w, wr);
    if (rc == PMGB_OK) rc = upload(ctx, &d_qxf, qxf);
    if (rc == PMGB_OK) rc = upload(ctx, &d_q, q);
    cudaError_t e = cudaSuccess;
    if (rc == PMGB_OK) e = dev_malloc(ctx, reinterpret_cast<void**>(&d_sk), 2 * sizeof(double) * n_r);
    if (rc == PMGB_OK && e == cudaSuccess) e = dev_malloc(ctx, reinterpret_cast<void**>(&d_skw), sizeof(float2) * n_r);
    if (rc == PMGB_OK && e == cudaSuccess)
        e = dev_malloc(ctx, reinterpret_cast<void**>(&d_table), std::max<size_t>(sizeof(double2) * table_len, 16));
    if (rc == PMGB_OK && e == cudaSuccess)
        e = pmgb_launch_structure_factor(d_qxf, d_q, n_uq, d_k, d_w, n_r, kmax, d_table, d_sk, d_skw, ctx->stream);
    if (rc == PMGB_OK && e == cudaSuccess)
        e = cudaMemcpyAsync(sk_host, d_sk, 2 * sizeof(double) * n_r, cudaMemcpyDeviceToHost, ctx->stream);
    void* tmp[] = {d_k, d_w, d_qxf, d_q, d_sk, d_skw, d_table};
    for (void* p : tmp) dev_free(ctx, p);
    if (rc != PMGB_OK) return rc;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "structure factor");
    return PMGB_OK;
}

// With S(k) known (sk: traversal order): the caller-order copy, and for replicated frameworks
// the k-vectors that can contribute.  S(k) of n_a x n_b x n_c copies of a cell vanishes unless
// n_d | k_d for every d (the sum over copies of e^{2 pi i k_d j / n_d} is zero otherwise), so
// those k-vectors add nothing.  The strides ks_d = gcd of k_d over the k-vectors whose |S(k)|
// exceeds 1e-10 max |S| (the others are FP64 rounding of an exact zero); the k-vectors that are
// not multiples are dropped if the most they could add, sum wt |S(k)| sum_g |q_g|, stays under
// 1e-9 K.  A framework that is not a replica keeps every k-vector (ks = 1).  Host only.
static void ewald_finish_host(const pmgb_system* s, const EwaldHost& eh, const double* sk, EwaldFinal& ef) {
    const int n_kvecs = eh.n_kvecs;
    const std::vector<int>& kabc = eh.kabc;
    const std::vector<double>& wt = eh.wt;
    ef.h_sk.assign(2 * static_cast<size_t>(n_kvecs), 0.0);
    for (int i = 0; i < n_kvecs; ++i) {
        ef.h_sk[2 * eh.order[i]] = sk[2 * i];
        ef.h_sk[2 * eh.order[i] + 1] = sk[2 * i + 1];
    }
    int* ks = ef.ks;
    {
        double smax = 0.0;
        for (int i = 0; i < n_kvecs; ++i) smax = std::max(smax, std::hypot(sk[2 * i], sk[2 * i + 1]));
        int g[3] = {0, 0, 0};
        for (int i = 0; i < n_kvecs; ++i)
            if (std::hypot(sk[2 * i], sk[2 * i + 1]) > 1e-10 * smax)
                for (int d = 0; d < 3; ++d) g[d] = std::gcd(g[d], std::abs(kabc[3 * i + d]));
        for (int d = 0; d < 3; ++d) ks[d] = g[d] > 0 ? g[d] : 1;
        double qg = 0.0;
        for (int k = 0; k < s->n_sites; ++k) qg += std::fabs(s->dev.q64[k]);
        double dropped = 0.0;
        for (int i = 0; i < n_kvecs; ++i)
            if (kabc[3 * i] % ks[0] || kabc[3 * i + 1] % ks[1] || kabc[3 * i + 2] % ks[2])
                dropped += std::fabs(wt[i]) * std::hypot(sk[2 * i], sk[2 * i + 1]) * qg;
        if (dropped > 1e-9) ks[0] = ks[1] = ks[2] = 1;
    }
    ef.pruned = ks[0] * ks[1] * ks[2] > 1;
    if (ef.pruned) {
        // kept k-vectors: the multiples, each half-row thinned to every ks2-th kc, rows in k / ks
        for (const KRow& r : eh.rows) {
            if (r.ka % ks[0] || r.kb % ks[1]) continue;
            KRow q{r.ka / ks[0], r.kb / ks[1], 0, 0, static_cast<int>(ef.wt.size()), r.dir, 0, 0};
            for (int m = 0; m < r.n; ++m) {
                const int kc = r.kc0 + r.dir * m;
                if (kc % ks[2]) continue;
                const int i = r.off + m;
                if (q.n == 0) q.kc0 = kc / ks[2];
                ++q.n;
                ef.kabc.insert(ef.kabc.end(), {r.ka, r.kb, kc});
                ef.wt.push_back(wt[i]);
                ef.sk.push_back(sk[2 * i]);
                ef.sk.push_back(sk[2 * i + 1]);
                ef.skw.push_back(make_float2(static_cast<float>(wt[i] * sk[2 * i]),
                                             static_cast<float>(wt[i] * sk[2 * i + 1])));
            }
            if (q.n > 0) ef.rows.push_back(q);
        }
    } else {
        ef.rows = eh.rows;
        ef.kabc = kabc;
        ef.wt = wt;
        ef.sk.assign(sk, sk + 2 * static_cast<size_t>(n_kvecs));
        for (int i = 0; i < n_kvecs; ++i)
            ef.skw.push_back(make_float2(static_cast<float>(wt[i] * sk[2 * i]), static_cast<float>(wt[i] * sk[2 * i + 1])));
    }
    const size_t n_eval = ef.wt.size();
    ef.tk.resize(n_eval);
    for (size_t i = 0; i < n_eval; ++i) {
        const float2 re = to_df(ef.wt[i] * ef.sk[2 * i]), im = to_df(ef.wt[i] * ef.sk[2 * i + 1]);
        ef.tk[i] = make_float4(re.x, re.y, im.x, im.y);
    }
}

// Device half after S(k): the kept k-vector arrays, the double-float weights, the rows and the
// shared erfc table; then every Ewald field of s->dev (asynchronous; no synchronisation).
static int ewald_upload_finish(pmgb_ctx* ctx, pmgb_system* s, EwaldHost& eh, EwaldFinal& ef) {
    int rc;
    if (ef.pruned || !s->d_sk) {  // (no device S(k) yet: it was evaluated from the unit cell)
        void* full[] = {s->d_skw, s->d_sk, s->d_kabc, s->d_wt};
        for (void* p : full) dev_free(ctx, p);
        s->d_skw = nullptr;
        s->d_sk = nullptr;
        s->d_kabc = nullptr;
        s->d_wt = nullptr;
        if ((rc = upload(ctx, &s->d_kabc, ef.kabc, &s->h2d_bytes)) ||
            (rc = upload(ctx, &s->d_wt, ef.wt, &s->h2d_bytes)) || (rc = upload(ctx, &s->d_sk, ef.sk, &s->h2d_bytes)) ||
            (rc = upload(ctx, &s->d_skw, ef.skw, &s->h2d_bytes)))
            return rc;
    }
    if ((rc = upload(ctx, &s->d_tk_df, ef.tk, &s->h2d_bytes))) return rc;
    if ((rc = upload(ctx, &s->d_krow, ef.rows, &s->h2d_bytes))) return rc;
    const pmgb_ctx::EsTable* es = nullptr;
    if ((rc = es_table_for(ctx, eh.alpha, eh.sr_cutoff * eh.sr_cutoff, &es))) return rc;
    const double alpha = eh.alpha, sr_cutoff = eh.sr_cutoff;
    s->n_k = eh.n_kvecs;
    s->k_order.swap(eh.order);
    s->h_sk.swap(ef.h_sk);
    s->ewald_set = true;
    for (int d = 0; d < 3; ++d) s->dev.ks[d] = ef.ks[d];
    s->dev.alpha = static_cast<float>(alpha);
    s->dev.rc2e = static_cast<float>(sr_cutoff * sr_cutoff);
    s->dev.alpha64 = alpha;
    s->dev.rc2e_64 = sr_cutoff * sr_cutoff;
    update_centre_image(s);
    s->dev.es_tab = es->d_es;
    s->dev.es_e_lo = PMGB_ES_E_LO;
    s->dev.es_n_oct = es->n / (PMGB_ES_COEF * PMGB_ES_SUB);
    s->dev.es_tab_df = es->d_es_df;
    s->dev.tk_df = s->d_tk_df;
    s->dev.rc2e_df = to_df(sr_cutoff * sr_cutoff);
    s->dev.sk64 = s->d_sk;
    s->dev.wt64 = s->d_wt;
    s->dev.kabc = s->d_kabc;
    s->dev.n_krow = static_cast<int>(ef.rows.size());
    s->dev.n_k = static_cast<int>(ef.wt.size());
    s->dev.krow = s->d_krow;
    s->dev.skw = s->d_skw;
    return PMGB_OK;
}

extern "C" int pmgb_system_set_ewald(pmgb_system* s, double alpha, double sr_cutoff, int32_t n_kvecs,
                                     const int32_t* kvec_abc, const double* kvec_wt) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    EwaldHost eh;
    Err er;
    if (ewald_build_host(alpha, sr_cutoff, n_kvecs, kvec_abc, kvec_wt, eh, er) != PMGB_OK)
        return fail(ctx, er.code, "%s", er.msg.c_str());
    PMGB_CK(ctx, enter_device(ctx->device));
    std::vector<double> sk(2 * static_cast<size_t>(n_kvecs));
    if (int rc = ewald_launch_sk(ctx, s, eh, sk.data())) return rc;
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    EwaldFinal ef;
    ewald_finish_host(s, eh, sk.data(), ef);
    if (int rc = ewald_upload_finish(ctx, s, eh, ef)) return rc;
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return PMGB_OK;
}

// Run body(i) for i in [0, n) on up to n_threads host threads (0: one per hardware thread).
template <class F>
static void run_parallel(int n, int n_threads, F body) {
    int t = n_threads > 0 ? n_threads : static_cast<int>(std::thread::hardware_concurrency());
    t = std::max(1, std::min({t, 64, n}));
    if (t == 1) {
        for (int i = 0; i < n; ++i) body(i);
        return;
    }
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    pool.reserve(t);
    for (int k = 0; k < t; ++k)
        pool.emplace_back([&] {
            for (int i = next++; i < n; i = next++) body(i);
        });
    for (auto& th : pool) th.join();
}

extern "C" int pmgb_systems_create_unitcell(pmgb_ctx* ctx, int32_t n_systems, const double* const* f_to_c,
                                            const int32_t* n_atoms, const double* const* atom_xf,
                                            const int32_t* const* atom_species, const int32_t* n_charges,
                                            const double* const* charge_xf, const double* const* charge_q,
                                            const int32_t* n_species, const double* const* epsilon,
                                            const double* const* sigma2, double r_cutoff, const int32_t* n_guest_atoms,
                                            const double* const* guest_atom_x, const int32_t* const* guest_atom_species,
                                            const int32_t* n_guest_charges, const double* const* guest_charge_x,
                                            const double* const* guest_charge_q, double ewald_precision,
                                            int32_t n_threads, int32_t* repfactors_out, pmgb_system** out) {
    if (!ctx) return PMGB_ERR_INVALID_ARGUMENT;
    const char* self = n_systems == 1 ? "pmgb_system_create_unitcell" : "pmgb_systems_create_unitcell";
    if (n_systems < 0 || !out ||
        (n_systems > 0 && (!f_to_c || !n_atoms || !atom_xf || !atom_species || !n_charges || !charge_xf ||
                           !charge_q || !n_species || !epsilon || !sigma2 || !n_guest_atoms || !guest_atom_x ||
                           !guest_atom_species || !n_guest_charges || !guest_charge_x || !guest_charge_q)))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "%s: bad arguments", self);
    for (int i = 0; i < n_systems; ++i) out[i] = nullptr;
    if (n_systems == 0) return PMGB_OK;
    struct Item {
        pmgb_system* s = nullptr;
        SysHost h;
        bool charged = false;
        EwaldHost eh;
        EwaldFinal ef;
        size_t sk_off = 0;
        int32_t rep[3] = {1, 1, 1};
        std::vector<int> unit_idx;  // S(k) from the unit cell: the k-vectors evaluated (traversal positions)
        Err er;
    };
    std::vector<Item> items(static_cast<size_t>(n_systems));
    for (Item& it : items) {
        it.s = new pmgb_system();
        it.s->ctx = ctx;
    }
    auto give_up = [&](int rc) {
        for (Item& it : items) {
            free_system_device(it.s);
            delete it.s;
        }
        return rc;
    };
    // host: supercell, records and, for charged pairs, the Ewald parameters and k-vector rows
    run_parallel(n_systems, n_threads, [&](int i) {
        Item& it = items[i];
        try {
            PmgbSupercell sc;
            const char* why = nullptr;
            if (pmgb_make_supercell(f_to_c[i], r_cutoff, n_atoms[i], atom_xf[i], atom_species[i], n_charges[i],
                                    charge_xf[i], charge_q[i], sc, &why) != PMGB_OK) {
                it.er.set(PMGB_ERR_INVALID_ARGUMENT, "%s", why);
                return;
            }
            for (int d = 0; d < 3; ++d) it.rep[d] = sc.rep[d];
            const CreateIn in{sc.f_to_c,
                              static_cast<int32_t>(sc.atom_species.size()),
                              sc.atom_xf.data(),
                              sc.atom_species.data(),
                              static_cast<int32_t>(sc.charge_q.size()),
                              sc.charge_xf.data(),
                              sc.charge_q.data(),
                              n_species[i],
                              epsilon[i],
                              sigma2[i],
                              r_cutoff * r_cutoff,
                              n_guest_atoms[i],
                              guest_atom_x[i],
                              guest_atom_species[i],
                              n_guest_charges[i],
                              guest_charge_x[i],
                              guest_charge_q[i]};
            if (system_build_host(in, it.s, it.h, it.er) != PMGB_OK) return;
            it.charged = n_charges[i] > 0 && n_guest_charges[i] > 0;  // src/henry.jl:93-97
            if (it.charged) {
                double alpha = 0.0;
                int64_t n_k = 0;
                std::vector<int32_t> abc;
                std::vector<double> wt;
                if (pmgb_ewald_kvectors(sc.f_to_c, r_cutoff, ewald_precision, &alpha, nullptr, nullptr, &abc, &wt,
                                        &n_k) != PMGB_OK ||
                    n_k > INT32_MAX) {
                    it.er.set(PMGB_ERR_INVALID_ARGUMENT, "Ewald set-up failed (precision must lie in (0, 1))");
                    return;
                }
                ewald_build_host(alpha, r_cutoff, static_cast<int32_t>(n_k), abc.data(), wt.data(), it.eh, it.er);
            }
        } catch (const std::bad_alloc&) {
            it.er.set(PMGB_ERR_OUT_OF_MEMORY, "host memory exhausted");
        }
    });
    for (int i = 0; i < n_systems; ++i)
        if (items[i].er.code != PMGB_OK) {
            const int code = items[i].er.code;
            if (n_systems == 1) fail(ctx, code, "%s: %s", self, items[i].er.msg.c_str());
            else fail(ctx, code, "%s: system %d: %s", self, i, items[i].er.msg.c_str());
            return give_up(code);
        }
    // device: every system's arrays, then S(k) of the charged ones, back to back
    cudaError_t e = enter_device(ctx->device);
    if (e != cudaSuccess) return give_up(cuda_fail(ctx, e, "cudaSetDevice"));
    size_t sk_total = 0;
    for (Item& it : items)
        if (it.charged) {
            it.sk_off = sk_total;
            sk_total += 2 * static_cast<size_t>(it.eh.n_kvecs);
        }
    double* sk = nullptr;  // pinned: the S(k) copies do not wait on one another
    if (sk_total > 0) {
        if (ctx->sk_host_cap < sk_total) {
            if (ctx->sk_host) cudaFreeHost(ctx->sk_host);
            ctx->sk_host = nullptr;
            ctx->sk_host_cap = 0;
            size_t cap = 4096;
            while (cap < sk_total) cap <<= 1;
            e = cudaMallocHost(reinterpret_cast<void**>(&ctx->sk_host), sizeof(double) * cap);
            if (e != cudaSuccess) return give_up(cuda_fail(ctx, e, "cudaMallocHost"));
            ctx->sk_host_cap = cap;
        }
        sk = ctx->sk_host;
    }
    auto finish = [&](int rc) {
        if (sk) cudaStreamSynchronize(ctx->stream);  // the copies into the landing buffer are done
        return rc == PMGB_OK ? rc : give_up(rc);
    };
    for (int i = 0; i < n_systems; ++i) {
        Item& it = items[i];
        int rc = system_upload(ctx, it.s, it.h);
        if (rc == PMGB_OK && it.charged) {
            // the supercell is an exact replica: its S(k) from the unit cell's charges
            if (it.rep[0] * it.rep[1] * it.rep[2] > 1)
                rc = ewald_launch_sk_unit(ctx, it.s, it.eh, it.rep, n_charges[i], charge_xf[i], charge_q[i],
                                          it.unit_idx, sk + it.sk_off);
            else
                rc = ewald_launch_sk(ctx, it.s, it.eh, sk + it.sk_off);
        }
        if (rc != PMGB_OK) return finish(rc);
        it.h = SysHost{};  // staged: the host arrays are no longer needed
    }
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return finish(cuda_fail(ctx, e, self));
    // host: the k-vectors kept once S(k) is known
    run_parallel(n_systems, n_threads, [&](int i) {
        Item& it = items[i];
        if (!it.charged) return;
        try {
            const double* skv = sk + it.sk_off;
            std::vector<double> full;
            const int n_img = it.rep[0] * it.rep[1] * it.rep[2];
            if (n_img > 1) {  // S(k) of every k-vector: n_img S_cell(k / rep) on the multiples, 0 elsewhere
                full.assign(2 * static_cast<size_t>(it.eh.n_kvecs), 0.0);
                for (size_t m = 0; m < it.unit_idx.size(); ++m) {
                    full[2 * it.unit_idx[m]] = n_img * skv[2 * m];
                    full[2 * it.unit_idx[m] + 1] = n_img * skv[2 * m + 1];
                }
                skv = full.data();
            }
            ewald_finish_host(it.s, it.eh, skv, it.ef);
        } catch (const std::bad_alloc&) {
            it.er.set(PMGB_ERR_OUT_OF_MEMORY, "host memory exhausted");
        }
    });
    for (int i = 0; i < n_systems; ++i)
        if (items[i].er.code != PMGB_OK) {
            fail(ctx, items[i].er.code, "%s: system %d: %s", self, i, items[i].er.msg.c_str());
            return finish(items[i].er.code);
        }
    for (Item& it : items)
        if (it.charged)
            if (int rc = ewald_upload_finish(ctx, it.s, it.eh, it.ef)) return finish(rc);
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return finish(cuda_fail(ctx, e, self));
    finish(PMGB_OK);
    for (int i = 0; i < n_systems; ++i) {
        ++ctx->refs;
        out[i] = items[i].s;
        if (repfactors_out)
            for (int d = 0; d < 3; ++d) repfactors_out[3 * i + d] = items[i].rep[d];
    }
    return PMGB_OK;
}

// Drop one reference to a system; the last one frees it (and releases its context).  Move handles
// and batches hold references, so a garbage-collected host may destroy the handles in any order.
// Errors of the teardown calls are cleared from the thread's CUDA error state, so that they are not
// reported later by an unrelated launch.
static void system_release(pmgb_system* s) {
    if (--s->refs > 0) return;
    pmgb_ctx* ctx = s->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    free_system_device(s);
    delete s;
    ctx_release(ctx);
    (void)cudaGetLastError();
}

extern "C" void pmgb_system_destroy(pmgb_system* s) {
    if (!s) return;
    system_release(s);
}

extern "C" int pmgb_system_info(const pmgb_system* s, int64_t* out6) {
    if (!s || !out6) return PMGB_ERR_INVALID_ARGUMENT;
    out6[0] = s->dev.n_rec;
    out6[1] = s->dev.n_seg;
    out6[2] = s->n_k;
    out6[3] = s->dev.n_k;
    out6[4] = s->n_sites;
    out6[5] = s->h2d_bytes;
    return PMGB_OK;
}

extern "C" int pmgb_system_n_sites(const pmgb_system* s) { return s ? s->n_sites : PMGB_ERR_INVALID_ARGUMENT; }

extern "C" int pmgb_system_sites(const pmgb_system* s, int32_t* site_atom, int32_t* site_charge) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < s->n_sites; ++k) {
        if (site_atom) site_atom[k] = s->site_atom[k];
        if (site_charge) site_charge[k] = s->site_charge[k];
    }
    return PMGB_OK;
}

extern "C" int pmgb_structure_factor(pmgb_system* s, double* sk_out) {
    if (!s || !sk_out) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    if (!s->ewald_set) return fail(ctx, PMGB_ERR_NOT_READY, "pmgb_structure_factor: Ewald parameters not set");
    std::copy(s->h_sk.begin(), s->h_sk.end(), sk_out);  // every caller k-vector, kept or not
    return PMGB_OK;
}

// ============================================================================
// launches
// ============================================================================
static int ready_for_charges(pmgb_system* s) {
    if (s->dev.charged && !s->ewald_set)
        return fail(s->ctx, PMGB_ERR_NOT_READY,
                    "framework and guest are charged: call pmgb_system_set_ewald before evaluating energies");
    return PMGB_OK;
}

static LaunchArgs base_args(pmgb_system* s) {
    LaunchArgs a{};
    a.sys = s->dev;
    a.status = s->ctx->d_status;
    return a;
}

static int sm_count(pmgb_ctx* ctx) {
    int n_sm = 0;
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, ctx->device);
    return std::max(1, n_sm);
}

// Chunk-items the double-float pass may need for n entries of this system: at most 4096 while
// the entries are cut finely, else n times the coarse chunk count (the refinement's rule).
static long long exact_items(const pmgb_system* s, int64_t n) {
    const long long work = static_cast<long long>(s->n_sites) * (s->dev.n_rec + (s->dev.charged ? s->dev.n_k : 0));
    const long long coarse = std::max(1ll, std::min(64ll, (work + 16383) / 16384));
    return std::max<long long>(4096, static_cast<long long>(n) * coarse);
}

// Refinement arguments and scratch for a double-float pass over up to n entries with n_screen
// screen chunks (0: every entry): entry list, screen counts and offsets (then the work counter),
// plan, per-entry chunk counts and chunk partials, from the system's grow-only buffers.
static int exact_args(pmgb_system* s, int64_t n, int n_screen, RefineArgs& r) {
    pmgb_ctx* ctx = s->ctx;
    const long long items = exact_items(s, n);
    int rc;
    if ((rc = ensure(ctx, s->r_list, sizeof(long long) * n)) ||
        (rc = ensure(ctx, s->r_counts, sizeof(int) * std::max(1, n_screen))) ||
        (rc = ensure(ctx, s->r_offsets, sizeof(int) * (n_screen + 2))) || (rc = ensure(ctx, s->r_plan, sizeof(int) * 4)) ||
        (rc = ensure(ctx, s->r_done, sizeof(int) * n)) || (rc = ensure(ctx, s->r_part, sizeof(double) * 4 * items)))
        return rc;
    r = RefineArgs{};
    r.sys = s->dev;
    r.n_systems = 1;
    r.n_blocks = 1;
    r.counts = static_cast<int*>(s->r_counts.p);
    r.offsets = static_cast<int*>(s->r_offsets.p);
    r.list = static_cast<long long*>(s->r_list.p);
    r.counter = r.offsets + n_screen + 1;
    r.plan = static_cast<int*>(s->r_plan.p);
    r.one_chunk = r.plan + 2;
    r.done = static_cast<int*>(s->r_done.p);
    r.part = static_cast<double*>(s->r_part.p);
    r.cap_items = items;
    r.cap_entries = n;
    s->last_refined_slot = n_screen;
    return PMGB_OK;
}

// Upload explicit site coordinates in FP64, each wrapped into [0, 1) (a whole-cell shift: the
// same minimum images), for the double-float pass.
static int upload_sites64(pmgb_system* s, size_t n_coord, const double* site_xf) {
    pmgb_ctx* ctx = s->ctx;
    std::vector<double> x(n_coord);
    for (size_t i = 0; i < n_coord; ++i) x[i] = wrap01(site_xf[i]);
    if (int rc = ensure(ctx, s->x64, sizeof(double) * n_coord)) return rc;
    PMGB_CK(ctx, cudaMemcpyAsync(s->x64.p, x.data(), sizeof(double) * n_coord, cudaMemcpyHostToDevice, ctx->stream));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));  // the staging vector is released on return
    return PMGB_OK;
}

// Enqueue double-float energies of n_conf configurations (coordinates in s->x64) into e_out_dev
// as (U_vdw, U_es short-range, U_es long-range).
static int exact_energies(pmgb_system* s, int64_t n_conf, double* e_out_dev) {
    pmgb_ctx* ctx = s->ctx;
    RefineArgs r;
    if (int rc = exact_args(s, n_conf, 0, r)) return rc;
    r.pose_src = REFINE_POSE_SITES;
    r.site_xf = static_cast<const double*>(s->x64.p);
    r.ref_u = e_out_dev;
    PMGB_CK(ctx, pmgb_launch_exact(r, n_conf, nullptr, sm_count(ctx), ctx->stream));
    return PMGB_OK;
}

extern "C" int pmgb_energies(pmgb_system* s, int64_t n_conf, const double* site_xf, double* out) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    if (n_conf < 0 || (n_conf > 0 && (!site_xf || !out)))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energies: bad arguments");
    if (int rc = ready_for_charges(s)) return rc;
    if (n_conf == 0) return PMGB_OK;
    if (n_conf > INT32_MAX)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energies: n_conf too large");
    PMGB_CK(ctx, enter_device(ctx->device));
    const size_t n_coord = 3 * static_cast<size_t>(s->n_sites) * static_cast<size_t>(n_conf);
    for (size_t i = 0; i < n_coord; ++i)
        if (!std::isfinite(site_xf[i]))
            return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energies: non-finite site coordinate at %zu", i);
    if (s->exact) {
        // every configuration in double-float from its FP64 coordinates
        int rc;
        if ((rc = upload_sites64(s, n_coord, site_xf)) ||
            (rc = ensure(ctx, s->out_buf, sizeof(double) * 3 * static_cast<size_t>(n_conf))) ||
            (rc = exact_energies(s, n_conf, static_cast<double*>(s->out_buf.p))))
            return rc;
        PMGB_CK(ctx, cudaMemcpyAsync(out, s->out_buf.p, sizeof(double) * 3 * static_cast<size_t>(n_conf),
                                     cudaMemcpyDeviceToHost, ctx->stream));
        return check_status(ctx);
    }
    std::vector<uint32_t> fix(n_coord);
    for (size_t i = 0; i < n_coord; ++i) fix[i] = to_fix(site_xf[i]);
    const size_t in_bytes = sizeof(uint32_t) * n_coord;
    const size_t out_bytes = sizeof(double) * 3 * static_cast<size_t>(n_conf);
    int rc;
    if ((rc = ensure(ctx, s->in_buf, in_bytes)) || (rc = ensure(ctx, s->out_buf, out_bytes))) return rc;
    PMGB_CK(ctx, cudaMemcpyAsync(s->in_buf.p, fix.data(), in_bytes, cudaMemcpyHostToDevice, ctx->stream));
    LaunchArgs a = base_args(s);
    a.pose_mode = POSE_SITES;
    a.out_mode = OUT_ENERGY;
    a.site_fix = static_cast<const uint32_t*>(s->in_buf.p);
    a.n_conf = n_conf;
    a.e_out = static_cast<double*>(s->out_buf.p);
    if (n_conf <= kLatencyConfs) {
        // few configurations (a Monte Carlo move): one CTA each, the framework split over its threads
        PMGB_CK(ctx, pmgb_launch_energies_latency(a, static_cast<int>(n_conf), ctx->stream));
    } else {
        const int n_ctas = static_cast<int>((n_conf + PMGB_THREADS - 1) / PMGB_THREADS);
        PMGB_CK(ctx, pmgb_launch_pairs(a, n_ctas, ctx->stream));
    }
    PMGB_CK(ctx, cudaMemcpyAsync(out, s->out_buf.p, out_bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return check_status(ctx);  // synchronises: the host staging vector outlives the copy
}

// ---------------------------------------------------------------------------- Monte Carlo moves
struct pmgb_move {
    pmgb_system* sys = nullptr;
    int max_conf = 0;
    bool exact = false;           // the system's exact setting when the handle was created
    // pinned staging: [0] = n_conf, then the site coordinates: 32-bit fixed point (FP32 pass)
    // or FP64 words (exact: the count in the first word's low 32 bits)
    void* h_stage = nullptr;
    double* h_out = nullptr;      // pinned: 3 per configuration
    void* d_stage = nullptr;
    double* d_out = nullptr;
    // the double-float pass's own scratch (the graph must not follow the system's buffers)
    long long* d_list = nullptr;
    int* d_offsets = nullptr;     // [0] entry count, [1] work counter
    int* d_plan = nullptr;
    int* d_done = nullptr;
    double* d_part = nullptr;
    cudaGraphExec_t exec = nullptr;
};

static void move_free(pmgb_move* m) {
    if (m->exec) cudaGraphExecDestroy(m->exec);
    if (m->h_stage) cudaFreeHost(m->h_stage);
    if (m->h_out) cudaFreeHost(m->h_out);
    void* dev[] = {m->d_stage, m->d_out, m->d_list, m->d_offsets, m->d_plan, m->d_done, m->d_part};
    for (void* p : dev)
        if (p) cudaFree(p);
}

extern "C" int pmgb_move_create(pmgb_system* s, int32_t max_conf, pmgb_move** out) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    if (!out || max_conf < 1 || max_conf > 65535)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_move_create: max_conf in [1, 65535]");
    if (int rc = ready_for_charges(s)) return rc;
    *out = nullptr;
    PMGB_CK(ctx, enter_device(ctx->device));
    auto* m = new pmgb_move();
    m->sys = s;
    m->max_conf = max_conf;
    m->exact = s->exact;
    const size_t words = 1 + static_cast<size_t>(max_conf) * s->n_sites * 3;
    const size_t stage_bytes = words * (m->exact ? sizeof(double) : sizeof(uint32_t));
    const long long items = exact_items(s, max_conf);
    cudaError_t e = cudaHostAlloc(&m->h_stage, stage_bytes, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&m->h_out), sizeof(double) * 3 * max_conf,
                                            cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaMalloc(&m->d_stage, stage_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&m->d_out, sizeof(double) * 3 * max_conf);
    if (m->exact) {
        if (e == cudaSuccess) e = cudaMalloc(&m->d_list, sizeof(long long) * max_conf);
        if (e == cudaSuccess) e = cudaMalloc(&m->d_offsets, sizeof(int) * 2);
        if (e == cudaSuccess) e = cudaMalloc(&m->d_plan, sizeof(int) * 4);
        if (e == cudaSuccess) e = cudaMalloc(&m->d_done, sizeof(int) * max_conf);
        if (e == cudaSuccess) e = cudaMalloc(&m->d_part, sizeof(double) * 4 * items);
    }
    if (e == cudaSuccess) {
        // one graph: copy in (count + coordinates), evaluate, copy out
        LaunchArgs a = base_args(s);
        a.pose_mode = POSE_SITES;
        a.out_mode = OUT_ENERGY;
        a.site_fix = static_cast<const uint32_t*>(m->d_stage) + 1;
        a.n_conf = max_conf;
        a.n_conf_dev = static_cast<const int*>(m->d_stage);
        a.e_out = m->d_out;
        RefineArgs r{};
        r.sys = s->dev;
        r.n_systems = 1;
        r.n_blocks = 1;
        r.offsets = m->d_offsets;
        r.counter = m->d_offsets + 1;
        r.list = m->d_list;
        r.plan = m->d_plan;
        r.one_chunk = m->d_plan + 2;
        r.done = m->d_done;
        r.part = m->d_part;
        r.cap_items = items;
        r.cap_entries = max_conf;
        r.pose_src = REFINE_POSE_SITES;
        r.site_xf = static_cast<const double*>(m->d_stage) + 1;
        r.ref_u = m->d_out;
        const int n_sm = sm_count(ctx);
        cudaStream_t st = ctx->stream;
        e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t e2 = cudaMemcpyAsync(m->d_stage, m->h_stage, stage_bytes, cudaMemcpyHostToDevice, st);
            if (e2 == cudaSuccess)
                e2 = m->exact ? pmgb_launch_exact(r, max_conf, a.n_conf_dev, n_sm, st)
                              : pmgb_launch_energies_latency(a, max_conf, st);
            if (e2 == cudaSuccess)
                e2 = cudaMemcpyAsync(m->h_out, m->d_out, sizeof(double) * 3 * max_conf, cudaMemcpyDeviceToHost, st);
            cudaGraph_t g = nullptr;
            e = cudaStreamEndCapture(st, &g);
            if (e == cudaSuccess) e = e2;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&m->exec, g, 0);
            if (g) cudaGraphDestroy(g);
        }
    }
    if (e != cudaSuccess) {
        move_free(m);
        delete m;
        return cuda_fail(ctx, e, "pmgb_move_create");
    }
    ++s->refs;  // the graph reads the system's device data: keep it alive with the handle
    *out = m;
    return PMGB_OK;
}

extern "C" int pmgb_move_energies(pmgb_move* m, int32_t n_conf, const double* site_xf, double* out) {
    if (!m) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = m->sys->ctx;
    if (n_conf < 0 || n_conf > m->max_conf || (n_conf > 0 && (!site_xf || !out)))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_move_energies: 0 <= n_conf <= %d", m->max_conf);
    if (n_conf == 0) return PMGB_OK;
    const size_t n_coord = 3 * static_cast<size_t>(m->sys->n_sites) * n_conf;
    for (size_t i = 0; i < n_coord; ++i)
        if (!std::isfinite(site_xf[i]))
            return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_move_energies: non-finite site coordinate at %zu", i);
    if (m->exact) {
        double* st = static_cast<double*>(m->h_stage);
        for (size_t i = 0; i < n_coord; ++i) st[1 + i] = wrap01(site_xf[i]);
        const int32_t cnt[2] = {n_conf, 0};
        std::memcpy(st, cnt, sizeof(cnt));
    } else {
        uint32_t* st = static_cast<uint32_t*>(m->h_stage);
        for (size_t i = 0; i < n_coord; ++i) st[1 + i] = to_fix(site_xf[i]);
        st[0] = static_cast<uint32_t>(n_conf);
    }
    PMGB_CK(ctx, enter_device(ctx->device));
    PMGB_CK(ctx, cudaGraphLaunch(m->exec, ctx->stream));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    std::memcpy(out, m->h_out, sizeof(double) * 3 * n_conf);
    return PMGB_OK;
}

extern "C" void pmgb_move_destroy(pmgb_move* m) {
    if (!m) return;
    pmgb_system* s = m->sys;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    move_free(m);
    delete m;
    system_release(s);
    (void)cudaGetLastError();
}

// Enqueue the FP64 refinement of the Boltzmann tail of a Widom run whose block results are
// in block_out_dev and per-insertion energies in u_dev (both corrected in place).  at_point
// (rotational energy grids): the run's poses sit at grid points (its pose fields are used).
static int run_refine(pmgb_system* s, int64_t n_per_block, int32_t n_blocks, uint64_t seed, double temperature,
                      double* block_out_dev, double* u_dev, double tail, const RefineArgs* at_point = nullptr) {
    pmgb_ctx* ctx = s->ctx;
    const int64_t cpb = (n_per_block + PMGB_THREADS - 1) / PMGB_THREADS;
    const int n_ctas = static_cast<int>(cpb * n_blocks);
    const int64_t n = n_per_block * n_blocks;
    int rc;
    if ((rc = ensure(ctx, s->r_hist, sizeof(unsigned long long) * pmgb_refine_hist_words() * n_blocks)) ||
        (rc = ensure(ctx, s->r_cut, sizeof(int) * n_blocks)) || (rc = ensure(ctx, s->r_counts, sizeof(int) * n_ctas)) ||
        (rc = ensure(ctx, s->r_offsets, sizeof(int) * (n_ctas + 2))) ||
        (rc = ensure(ctx, s->r_list, sizeof(long long) * n)) || (rc = ensure(ctx, s->r_ref, sizeof(double) * 3 * n)) ||
        (rc = ensure(ctx, s->r_plan, sizeof(int) * 4)) || (rc = ensure(ctx, s->r_done, sizeof(int) * n)) ||
        (rc = ensure(ctx, s->r_part, sizeof(double) * 4 * (2 * n + 4096))))
        return rc;
    RefineArgs r{};
    r.sys = s->dev;
    r.n_systems = 1;
    r.n_per_block = n_per_block;
    r.n_blocks = n_blocks;
    r.ctas_per_block = static_cast<int>(cpb);
    r.seed = seed;
    r.inv_temperature = 1.0 / temperature;
    r.tail = tail;
    if (at_point) {
        r.pose_src = REFINE_POSE_ROTGRID;
        for (int d = 0; d < 3; ++d) {
            r.grid_n[d] = at_point->grid_n[d];
            r.grid_rep[d] = at_point->grid_rep[d];
        }
        r.grid_ax64 = at_point->grid_ax64;
        r.point_base = at_point->point_base;
        r.item_base = at_point->item_base;
    }
    r.block_out = block_out_dev;
    r.partials = static_cast<LsePartial*>(s->partials.p);
    r.u = u_dev;
    r.hist = static_cast<unsigned long long*>(s->r_hist.p);
    r.cut = static_cast<int*>(s->r_cut.p);
    r.counts = static_cast<int*>(s->r_counts.p);
    r.offsets = static_cast<int*>(s->r_offsets.p);
    r.list = static_cast<long long*>(s->r_list.p);
    r.ref_u = static_cast<double*>(s->r_ref.p);
    r.counter = static_cast<int*>(s->r_offsets.p) + n_ctas + 1;
    r.plan = static_cast<int*>(s->r_plan.p);
    r.one_chunk = r.plan + 2;
    r.done = static_cast<int*>(s->r_done.p);
    r.part = static_cast<double*>(s->r_part.p);
    r.cap_entries = n;
    r.cap_items = 2 * n + 4096;
    int n_sm = 0;
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, ctx->device);
    PMGB_CK(ctx, pmgb_launch_refine(r, n_ctas, std::max(1, n_sm), ctx->stream));
    s->last_refined_slot = n_ctas;
    return PMGB_OK;
}

extern "C" int pmgb_system_refined_count(pmgb_system* s, int64_t* count_out) {
    if (!s || !count_out) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    *count_out = 0;
    if (s->last_refined_slot < 0) return PMGB_OK;
    PMGB_CK(ctx, enter_device(ctx->device));
    int n = 0;
    PMGB_CK(ctx, cudaMemcpyAsync(&n, static_cast<int*>(s->r_offsets.p) + s->last_refined_slot, sizeof(int),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    *count_out = n;
    return PMGB_OK;
}

extern "C" int pmgb_system_set_accessibility(pmgb_system* s, const int32_t n_pts[3], const int32_t repfactors[3],
                                             const uint8_t* data) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    if (!data) {
        s->dev.acc = nullptr;
        return PMGB_OK;
    }
    if (!n_pts || !repfactors)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_system_set_accessibility: n_pts and repfactors required");
    for (int d = 0; d < 3; ++d)
        if (n_pts[d] < 1 || repfactors[d] < 1)
            return fail(ctx, PMGB_ERR_INVALID_ARGUMENT,
                        "pmgb_system_set_accessibility: n_pts and repfactors must be >= 1");
    const size_t n = static_cast<size_t>(n_pts[0]) * n_pts[1] * n_pts[2];
    PMGB_CK(ctx, enter_device(ctx->device));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));  // no run may still read the old grid
    if (int rc = ensure(ctx, s->acc, n)) return rc;
    std::vector<uint8_t> h(data, data + n);
    for (auto& v : h) v = v ? 1 : 0;
    PMGB_CK(ctx, cudaMemcpyAsync(s->acc.p, h.data(), n, cudaMemcpyHostToDevice, ctx->stream));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    s->dev.acc = static_cast<const uint8_t*>(s->acc.p);
    for (int d = 0; d < 3; ++d) {
        s->dev.acc_n[d] = n_pts[d];
        s->dev.acc_rep[d] = repfactors[d];
    }
    return PMGB_OK;
}

extern "C" int pmgb_system_set_cull(pmgb_system* s, int32_t on) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    s->cull = on != 0;
    return PMGB_OK;
}

extern "C" int pmgb_system_set_image_lists(pmgb_system* s, int32_t mode) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    if (mode < 0 || mode > 2)
        return fail(s->ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_system_set_image_lists: mode 0 (off), 1 (auto) or 2 (on)");
    s->image_lists = mode;
    return PMGB_OK;
}

// Whether the spatially ordered forward Widom pass of a run of n insertions takes image lists: a
// guest form the kernels instantiate, every perpendicular width above twice the larger cutoff (at
// most one image of a record within the cutoff of a site; the replication factors guarantee it for
// the LJ cutoff), and (auto) a CTA's list expected to be short enough to pay.  The CTA's 256
// insertions, consecutive along the run's Hilbert order, occupy about 256 V / n of the cell: a
// region of radius ~1.6 (3 256 V / (4 pi n))^(1/3) (from simulated orders of the config1, config3
// and config4 shapes); its list holds the images within cutoff + guest reach + that radius of the
// centre.  Measured on GB300: a run of one system gains below ~0.9 of the records when it fills
// the GPU (two CTAs per SM; a smaller grid leaves the list building exposed), a batch, which fills
// the GPU with many systems, below ~1.4.
static bool image_lists_fit(const pmgb_system* s, int mode) {
    if (mode == 0 || !pmgb_img_supported(s->dev.n_sites)) return false;
    const double rc2 = std::max<double>(s->dev.rc2, s->dev.charged ? s->dev.rc2e : 0.0);
    for (int a = 0; a < 3; ++a) {
        const double w = static_cast<double>(s->dev.cw[a]) * 4294967296.0;
        if (!(4.0 * rc2 < w * w * (1.0 - 1e-6))) return false;
    }
    return true;
}

static bool image_lists_for(const pmgb_system* s, int64_t n_insertions, bool in_batch) {
    if (!image_lists_fit(s, s->image_lists)) return false;
    if (s->image_lists == 2) return true;
    const double pi = 3.14159265358979323846;
    const double vol = std::fabs(s->dev.f2c64[0] * s->dev.f2c64[3] * s->dev.f2c64[5]);
    const double r_cta = 1.6 * std::cbrt(3.0 * PMGB_THREADS * vol / (4.0 * pi * std::max<int64_t>(n_insertions, 1)));
    const double rc = std::sqrt(std::max<double>(s->dev.rc2, s->dev.charged ? s->dev.rc2e : 0.0));
    const double reach = rc + s->dev.com_reach + r_cta;
    const double list = 4.0 / 3.0 * pi * reach * reach * reach / vol;  // expected list / records
    if (in_batch) return list < 1.4;
    const int64_t n_ctas = (n_insertions + PMGB_THREADS - 1) / PMGB_THREADS;
    return list < 0.9 && n_ctas >= 2 * static_cast<int64_t>(sm_count(s->ctx));
}

static bool uses_image_lists(const pmgb_system* s, int64_t n_insertions) {
    return s->cull && image_lists_for(s, n_insertions, false);
}

extern "C" int pmgb_system_image_lists(const pmgb_system* s, int64_t n_insertions, int32_t* on_out) {
    if (!s || !on_out || n_insertions < 1) return PMGB_ERR_INVALID_ARGUMENT;
    *on_out = uses_image_lists(s, n_insertions) ? 1 : 0;
    return PMGB_OK;
}

extern "C" int pmgb_system_centre_image(const pmgb_system* s, int32_t* on_out) {
    if (!s || !on_out) return PMGB_ERR_INVALID_ARGUMENT;
    *on_out = (s->dev.com_axis >= -1 && s->dev.n_sites > 1) ? 1 : 0;
    return PMGB_OK;
}

extern "C" int pmgb_system_kspace_mirror(const pmgb_system* s, int32_t* on_out) {
    if (!s || !on_out) return PMGB_ERR_INVALID_ARGUMENT;
    *on_out = s->dev.k_mirror;
    return PMGB_OK;
}

extern "C" int pmgb_system_set_centre_image(pmgb_system* s, int32_t on) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    s->centre_image = on != 0;
    update_centre_image(s);
    return PMGB_OK;
}

extern "C" int pmgb_system_set_exact(pmgb_system* s, int32_t on) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    s->exact = on != 0;
    return PMGB_OK;
}

extern "C" int pmgb_system_set_refine(pmgb_system* s, double tail_fraction) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    if (!(tail_fraction >= 0.0 && tail_fraction < 1.0))
        return fail(s->ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_system_set_refine: tail fraction in [0, 1)");
    s->refine_tail = tail_fraction;
    return PMGB_OK;
}

extern "C" int pmgb_widom_device(pmgb_system* s, int64_t n_per_block, int32_t n_blocks, uint64_t seed,
                                 double temperature, double* block_out_dev, double* u_out_dev) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    if (n_per_block < 1 || n_blocks < 1 || !block_out_dev)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom: need n_per_block >= 1, n_blocks >= 1, block_out");
    if (!(temperature > 0.0) || !std::isfinite(temperature))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom: temperature must be positive (got %g)", temperature);
    if (int rc = ready_for_charges(s)) return rc;
    // compare before multiplying: n_per_block near INT64_MAX must not wrap the CTA count
    if (n_per_block > static_cast<int64_t>(INT32_MAX) * PMGB_THREADS)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom: too many insertions per block for one launch");
    const int64_t cpb = (n_per_block + PMGB_THREADS - 1) / PMGB_THREADS;
    if (cpb > INT32_MAX / n_blocks)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom: too many insertions for one launch");
    PMGB_CK(ctx, enter_device(ctx->device));
    const int n_ctas = static_cast<int>(cpb * n_blocks);
    if (int rc = ensure(ctx, s->partials, sizeof(LsePartial) * n_ctas)) return rc;
    LaunchArgs a = base_args(s);
    a.pose_mode = POSE_PHILOX;
    a.out_mode = OUT_WIDOM;
    a.seed = seed;
    a.n_per_block = n_per_block;
    a.n_blocks = n_blocks;
    a.ctas_per_block = static_cast<int>(cpb);
    a.inv_temperature = 1.0 / temperature;
    a.partials = static_cast<LsePartial*>(s->partials.p);
    a.u_out = u_out_dev;
    const bool refine = s->refine_tail > 0.0;
    a.no_resid = refine ? 1 : 0;  // the refinement re-evaluates the insertions that matter in FP64
    const size_t n_ins = static_cast<size_t>(n_per_block) * n_blocks;
    if ((refine || s->cull) && !u_out_dev) {  // both need every insertion's FP32 energy
        if (int rc = ensure(ctx, s->g_u, sizeof(double) * 2 * n_ins)) return rc;
        a.u_out = static_cast<double*>(s->g_u.p);
    }
    if (uses_image_lists(s, static_cast<int64_t>(n_ins))) {
        // one spatial order over the whole run; warps gather their image lists (csrc/pmgb_img.cu);
        // the block sums are formed from the energies in insertion order
        if (n_ins > static_cast<size_t>(INT32_MAX))
            return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom: too many insertions for one run");
        const long long n_cells = 1ll << (3 * pmgb_run_order_bits(static_cast<long long>(n_ins)));
        int rc;
        if ((rc = ensure(ctx, s->o_counts, sizeof(int) * n_cells)) || (rc = ensure(ctx, s->o_perm, sizeof(int) * n_ins)))
            return rc;
        a.perm = static_cast<const int*>(s->o_perm.p);
        PMGB_CK(ctx, pmgb_launch_run_order(seed, static_cast<long long>(n_ins), static_cast<int*>(s->o_counts.p),
                                           static_cast<int*>(s->o_perm.p), ctx->stream));
        PMGB_CK(ctx, launch_pairs_timed(ctx, a, n_ctas, true));
        PMGB_CK(ctx, pmgb_launch_lse_from_u(a.u_out, n_per_block, n_blocks, a.ctas_per_block, a.inv_temperature,
                                            a.partials, ctx->stream));
    } else if (s->cull) {
        // spatially sorted processing order, so that warps can skip out-of-cutoff records; the
        // block sums are then formed from the energies in insertion order
        int rc;
        if ((rc = ensure(ctx, s->o_counts, sizeof(int) * pmgb_widom_order_cells() * n_blocks)) ||
            (rc = ensure(ctx, s->o_perm, sizeof(int) * n_ins)))
            return rc;
        a.perm = static_cast<const int*>(s->o_perm.p);
        PMGB_CK(ctx, pmgb_launch_widom_order(seed, n_per_block, n_blocks, static_cast<int*>(s->o_counts.p),
                                             static_cast<int*>(s->o_perm.p), ctx->stream));
        PMGB_CK(ctx, launch_pairs_timed(ctx, a, n_ctas));
        PMGB_CK(ctx, pmgb_launch_lse_from_u(a.u_out, n_per_block, n_blocks, a.ctas_per_block, a.inv_temperature,
                                            a.partials, ctx->stream));
    } else {
        PMGB_CK(ctx, launch_pairs_timed(ctx, a, n_ctas));
    }
    PMGB_CK(ctx, pmgb_launch_reduce_blocks(a.partials, n_blocks, a.ctas_per_block, block_out_dev, ctx->stream));
    if (refine) return run_refine(s, n_per_block, n_blocks, seed, temperature, block_out_dev, a.u_out, s->refine_tail);
    return PMGB_OK;
}

// The unordered FP32 Widom pass (per-site distances), with the per-CTA partials in the
// library's fixed device array instead of memory the system allocates; nothing is allocated
// or freed.  Spatial ordering with per-site distances changes no result bit (the ordered pass
// forms the same sums); image lists change FP32 roundings.  A system with FP64 tail refinement
// is refused.
extern "C" int pmgb_widom_noalloc(pmgb_system* s, int64_t n_per_block, int32_t n_blocks, uint64_t seed,
                                  double temperature, double* block_out_dev, double* u_out_dev) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    if (n_per_block < 1 || n_blocks < 1 || !block_out_dev)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT,
                    "pmgb_widom_noalloc: need n_per_block >= 1, n_blocks >= 1 and a device block_out");
    if (!(temperature > 0.0) || !std::isfinite(temperature))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom_noalloc: temperature must be positive (got %g)",
                    temperature);
    if (int rc = ready_for_charges(s)) return rc;
    if (s->refine_tail > 0.0)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT,
                    "pmgb_widom_noalloc: this system refines its Boltzmann tail in FP64 (pmgb_system_set_refine), "
                    "which needs per-run scratch the fixed array does not hold; switch refinement off for this "
                    "call or use pmgb_widom_device");
    // compare before multiplying: the CTA count must not wrap for huge n_per_block
    const int64_t cpb = (n_per_block + PMGB_THREADS - 1) / PMGB_THREADS;
    if (n_per_block > static_cast<int64_t>(PMGB_NOALLOC_MAX_CTAS) * PMGB_THREADS ||
        cpb > PMGB_NOALLOC_MAX_CTAS / n_blocks)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT,
                    "pmgb_widom_noalloc: %lld blocks of %lld insertions need more than the fixed scratch's %d CTAs "
                    "of %d insertions (at most %lld insertions per call)",
                    static_cast<long long>(n_blocks), static_cast<long long>(n_per_block), PMGB_NOALLOC_MAX_CTAS,
                    PMGB_THREADS, static_cast<long long>(PMGB_NOALLOC_MAX_CTAS) * PMGB_THREADS);
    PMGB_CK(ctx, enter_device(ctx->device));
    LsePartial* scratch = nullptr;
    PMGB_CK(ctx, pmgb_noalloc_scratch(ctx->device, &scratch));
    LaunchArgs a = base_args(s);
    a.pose_mode = POSE_PHILOX;
    a.out_mode = OUT_WIDOM;
    a.seed = seed;
    a.n_per_block = n_per_block;
    a.n_blocks = n_blocks;
    a.ctas_per_block = static_cast<int>(cpb);
    a.inv_temperature = 1.0 / temperature;
    a.partials = scratch;  // every entry the reduction reads is written by this launch first
    a.u_out = u_out_dev;
    PMGB_CK(ctx, pmgb_launch_pairs(a, static_cast<int>(cpb * n_blocks), ctx->stream));
    PMGB_CK(ctx, pmgb_launch_reduce_blocks(a.partials, n_blocks, a.ctas_per_block, block_out_dev, ctx->stream));
    return PMGB_OK;
}

extern "C" int pmgb_widom(pmgb_system* s, int64_t n_per_block, int32_t n_blocks, uint64_t seed, double temperature,
                          double* block_out, double* u_out) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    if (!block_out) return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom: block_out is NULL");
    if (n_per_block < 1 || n_blocks < 1)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom: need n_per_block >= 1 and n_blocks >= 1");
    PMGB_CK(ctx, enter_device(ctx->device));
    int rc;
    if ((rc = ensure(ctx, s->block_out, sizeof(double) * 4 * n_blocks))) return rc;
    const size_t u_bytes = u_out ? sizeof(double) * 2 * static_cast<size_t>(n_per_block) * n_blocks : 0;
    if (u_out && (rc = ensure(ctx, s->out_buf, u_bytes))) return rc;
    rc = pmgb_widom_device(s, n_per_block, n_blocks, seed, temperature, static_cast<double*>(s->block_out.p),
                           u_out ? static_cast<double*>(s->out_buf.p) : nullptr);
    if (rc) return rc;
    PMGB_CK(ctx, cudaMemcpyAsync(block_out, s->block_out.p, sizeof(double) * 4 * n_blocks, cudaMemcpyDeviceToHost,
                                 ctx->stream));
    if (u_out) PMGB_CK(ctx, cudaMemcpyAsync(u_out, s->out_buf.p, u_bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return check_status(ctx);
}

// ---------------------------------------------------------------------------- adjoint
static int grid_axes(pmgb_system* s, const int32_t n_pts[3], const int32_t rep[3]);
static int exact_grid(pmgb_system* s, const int32_t n_pts[3], const int32_t repfactors[3], double unit_factor,
                      float* out_dev);
static int template_sites(int n) { return n <= 1 ? 1 : n <= 2 ? 2 : n <= 3 ? 3 : n <= 4 ? 4 : n <= 6 ? 6 : 8; }

// Assemble Σ w ∂U/∂ε_ab and Σ w ∂U/∂σ²_ab (a: guest species, b: framework species) from the
// per (segment, site) weighted sums of r^-12 and r^-6:  U = 4ε(σ^12 r^-12 - σ^6 r^-6).
static void assemble_species(const pmgb_system* s, int nst, const double* cols, double* dtheta) {
    const int n = s->n_species;
    for (int i = 0; i < 2 * n * n; ++i) dtheta[3 + i] = 0.0;
    for (size_t sg = 0; sg < s->seg_species.size(); ++sg) {
        const int b = s->seg_species[sg];
        if (b < 0) continue;
        for (int k = 0; k < s->n_sites; ++k) {
            const int ga = s->site_species[k];
            if (ga < 0) continue;
            const double i12 = cols[(sg * nst + k) * 2], i6 = cols[(sg * nst + k) * 2 + 1];
            const double s2 = s->sig2[ga * n + b], e = s->eps[ga * n + b];
            const double s4 = s2 * s2, s6 = s4 * s2, s10 = s6 * s4, s12 = s6 * s6;
            dtheta[3 + 2 * (ga * n + b)] += 4.0 * (s12 * i12 - s6 * i6);
            dtheta[3 + 2 * (ga * n + b) + 1] += 4.0 * e * (6.0 * s10 * i12 - 3.0 * s4 * i6);
        }
    }
}

extern "C" int pmgb_widom_adjoint(pmgb_system* s, int64_t n_per_block, int32_t n_blocks, uint64_t seed,
                                  double temperature, double* block_out, double* dtheta, double* u_out,
                                  float* grad_out) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    if (n_per_block < 1 || n_blocks < 1 || !block_out || !dtheta)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom_adjoint: bad arguments");
    if (!(temperature > 0.0) || !std::isfinite(temperature))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom_adjoint: temperature must be positive");
    if (int rc = ready_for_charges(s)) return rc;
    // compare before multiplying: n_per_block near INT64_MAX must not wrap the CTA count
    if (n_per_block > static_cast<int64_t>(INT32_MAX) * PMGB_THREADS)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom_adjoint: too many insertions per block");
    const int64_t cpb = (n_per_block + PMGB_THREADS - 1) / PMGB_THREADS;
    if (cpb > INT32_MAX / n_blocks) return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom_adjoint: too many insertions");
    const int nst = template_sites(s->n_sites);
    const int n_cols = static_cast<int>(s->seg_species.size()) * nst * 2;
    const int64_t n = n_per_block * n_blocks;
    PMGB_CK(ctx, enter_device(ctx->device));
    const int n_ctas = static_cast<int>(cpb * n_blocks);
    const int n_chunks = static_cast<int>(std::min<int64_t>(1024, (n + 4095) / 4096));
    int rc;
    if ((rc = ensure(ctx, s->partials, sizeof(LsePartial) * n_ctas)) ||
        (rc = ensure(ctx, s->block_out, sizeof(double) * 4 * n_blocks)) ||
        (rc = ensure(ctx, s->g_u, sizeof(double) * 2 * n)) ||
        (rc = ensure(ctx, s->g_dsum, sizeof(float) * std::max<int64_t>(1, n_cols) * n)) ||
        (rc = ensure(ctx, s->g_part, sizeof(double) * n_chunks * (n_cols + 2))) ||
        (rc = ensure(ctx, s->g_cols, sizeof(double) * (n_cols + 2))) ||
        (grad_out && (rc = ensure(ctx, s->g_grad, sizeof(float) * 3 * n))))
        return rc;
    LaunchArgs a = base_args(s);
    a.pose_mode = POSE_PHILOX;
    a.out_mode = OUT_WIDOM;
    a.seed = seed;
    a.n_per_block = n_per_block;
    a.n_blocks = n_blocks;
    a.ctas_per_block = static_cast<int>(cpb);
    a.inv_temperature = 1.0 / temperature;
    a.partials = static_cast<LsePartial*>(s->partials.p);
    a.u_out = static_cast<double*>(s->g_u.p);
    a.dsum = static_cast<float*>(s->g_dsum.p);
    a.dsum_stride = n;
    a.grad_u = grad_out ? static_cast<float*>(s->g_grad.p) : nullptr;
    double* d_block = static_cast<double*>(s->block_out.p);
    if (!grad_out && uses_image_lists(s, n)) {
        // the forward pass's image lists, with the columns (no forces requested): one spatial
        // order over the whole run, block sums from the energies in insertion order
        if (n > INT32_MAX) return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom_adjoint: too many insertions for one run");
        const long long n_cells = 1ll << (3 * pmgb_run_order_bits(static_cast<long long>(n)));
        if ((rc = ensure(ctx, s->o_counts, sizeof(int) * n_cells)) || (rc = ensure(ctx, s->o_perm, sizeof(int) * n)))
            return rc;
        a.perm = static_cast<const int*>(s->o_perm.p);
        PMGB_CK(ctx, pmgb_launch_run_order(seed, static_cast<long long>(n), static_cast<int*>(s->o_counts.p),
                                           static_cast<int*>(s->o_perm.p), ctx->stream));
        PMGB_CK(ctx, pmgb_launch_pairs_img(a, n_ctas, ctx->stream));
        PMGB_CK(ctx, pmgb_launch_lse_from_u(a.u_out, n_per_block, n_blocks, a.ctas_per_block, a.inv_temperature,
                                            a.partials, ctx->stream));
    } else if (s->cull) {  // spatially ordered, block sums from the energies in insertion order
        if ((rc = ensure(ctx, s->o_counts, sizeof(int) * pmgb_widom_order_cells() * n_blocks)) ||
            (rc = ensure(ctx, s->o_perm, sizeof(int) * n)))
            return rc;
        a.perm = static_cast<const int*>(s->o_perm.p);
        PMGB_CK(ctx, pmgb_launch_widom_order(seed, n_per_block, n_blocks, static_cast<int*>(s->o_counts.p),
                                             static_cast<int*>(s->o_perm.p), ctx->stream));
        PMGB_CK(ctx, pmgb_launch_pairs_grad(a, n_ctas, ctx->stream));
        PMGB_CK(ctx, pmgb_launch_lse_from_u(a.u_out, n_per_block, n_blocks, a.ctas_per_block, a.inv_temperature,
                                            a.partials, ctx->stream));
    } else {
        PMGB_CK(ctx, pmgb_launch_pairs_grad(a, n_ctas, ctx->stream));
    }
    PMGB_CK(ctx, pmgb_launch_reduce_blocks(a.partials, n_blocks, a.ctas_per_block, d_block, ctx->stream));
    PMGB_CK(ctx, pmgb_launch_weighted_columns(a.u_out, 2, n, a.inv_temperature, d_block, n_blocks, a.dsum, n_cols, n,
                                              static_cast<double*>(s->g_part.p), n_chunks,
                                              static_cast<double*>(s->g_cols.p), ctx->stream));
    std::vector<double> cols(n_cols + 2), fp32_blocks(4 * static_cast<size_t>(n_blocks));
    // the column weights are relative to the FP32 block sums: keep those for M
    PMGB_CK(ctx, cudaMemcpyAsync(fp32_blocks.data(), d_block, sizeof(double) * 4 * n_blocks, cudaMemcpyDeviceToHost,
                                 ctx->stream));
    if (s->refine_tail > 0.0)
        if ((rc = run_refine(s, n_per_block, n_blocks, seed, temperature, d_block, a.u_out, s->refine_tail))) return rc;
    PMGB_CK(ctx, cudaMemcpyAsync(block_out, d_block, sizeof(double) * 4 * n_blocks, cudaMemcpyDeviceToHost, ctx->stream));
    PMGB_CK(ctx, cudaMemcpyAsync(cols.data(), s->g_cols.p, sizeof(double) * (n_cols + 2), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    if (u_out) PMGB_CK(ctx, cudaMemcpyAsync(u_out, a.u_out, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (grad_out) PMGB_CK(ctx, cudaMemcpyAsync(grad_out, a.grad_u, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
    if ((rc = check_status(ctx))) return rc;
    double M = -INFINITY;
    for (int b = 0; b < n_blocks; ++b) M = std::max(M, fp32_blocks[4 * b]);
    dtheta[0] = M;
    dtheta[1] = cols[n_cols];
    dtheta[2] = cols[n_cols + 1];
    assemble_species(s, nst, cols.data(), dtheta);
    return PMGB_OK;
}

extern "C" int pmgb_energies_grad(pmgb_system* s, int64_t n_conf, const double* site_xf, double* out,
                                  float* grad_out) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    if (n_conf < 0 || (n_conf > 0 && (!site_xf || !out || !grad_out)))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energies_grad: bad arguments");
    if (int rc = ready_for_charges(s)) return rc;
    if (n_conf == 0) return PMGB_OK;
    if (n_conf > INT32_MAX) return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energies_grad: n_conf too large");
    PMGB_CK(ctx, enter_device(ctx->device));
    const size_t n_coord = 3 * static_cast<size_t>(s->n_sites) * static_cast<size_t>(n_conf);
    std::vector<uint32_t> fix(n_coord);
    for (size_t i = 0; i < n_coord; ++i) {
        if (!std::isfinite(site_xf[i])) return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "non-finite site coordinate");
        fix[i] = to_fix(site_xf[i]);
    }
    const int nst = template_sites(s->n_sites);
    const int n_cols = static_cast<int>(s->seg_species.size()) * nst * 2;
    int rc;
    if ((rc = ensure(ctx, s->in_buf, sizeof(uint32_t) * n_coord)) || (rc = ensure(ctx, s->out_buf, sizeof(double) * 3 * n_conf)) ||
        (rc = ensure(ctx, s->g_grad, sizeof(float) * 3 * n_conf)) ||
        (rc = ensure(ctx, s->g_dsum, sizeof(float) * std::max(1, n_cols) * n_conf)))
        return rc;
    PMGB_CK(ctx, cudaMemcpyAsync(s->in_buf.p, fix.data(), sizeof(uint32_t) * n_coord, cudaMemcpyHostToDevice, ctx->stream));
    LaunchArgs a = base_args(s);
    a.pose_mode = POSE_SITES;
    a.out_mode = OUT_ENERGY;
    a.site_fix = static_cast<const uint32_t*>(s->in_buf.p);
    a.n_conf = n_conf;
    a.e_out = static_cast<double*>(s->out_buf.p);
    a.dsum = static_cast<float*>(s->g_dsum.p);
    a.dsum_stride = n_conf;
    a.grad_u = static_cast<float*>(s->g_grad.p);
    PMGB_CK(ctx, pmgb_launch_pairs_grad(a, static_cast<int>((n_conf + PMGB_THREADS - 1) / PMGB_THREADS), ctx->stream));
    // the energies to the FP64 tolerance (the gradients stay FP32)
    if (s->exact && ((rc = upload_sites64(s, n_coord, site_xf)) || (rc = exact_energies(s, n_conf, a.e_out))))
        return rc;
    PMGB_CK(ctx, cudaMemcpyAsync(out, s->out_buf.p, sizeof(double) * 3 * n_conf, cudaMemcpyDeviceToHost, ctx->stream));
    PMGB_CK(ctx, cudaMemcpyAsync(grad_out, s->g_grad.p, sizeof(float) * 3 * n_conf, cudaMemcpyDeviceToHost, ctx->stream));
    return check_status(ctx);
}

extern "C" int pmgb_energy_grid_adjoint(pmgb_system* s, const int32_t n_pts[3], const int32_t repfactors[3],
                                        double unit_factor, double temperature, float* out, float* grad_out,
                                        double* dtheta) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    if (!n_pts || !repfactors || !out || !dtheta || !(temperature > 0.0))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energy_grid_adjoint: bad arguments");
    for (int d = 0; d < 3; ++d)
        if (n_pts[d] < 1 || repfactors[d] < 1)
            return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energy_grid_adjoint: n_pts and repfactors must be >= 1");
    if (s->n_sites != 1)
        return fail(ctx, PMGB_ERR_UNSUPPORTED, "pmgb_energy_grid_adjoint: the probe must be a single site");
    const int64_t total = int64_t(n_pts[0]) * n_pts[1] * n_pts[2];
    PMGB_CK(ctx, enter_device(ctx->device));
    if (int rc = grid_axes(s, n_pts, repfactors)) return rc;
    const int n_cols = static_cast<int>(s->seg_species.size()) * 1 * 2;
    const int n_chunks = static_cast<int>(std::min<int64_t>(1024, (total + 4095) / 4096));
    int rc;
    if ((rc = ensure(ctx, s->out_buf, sizeof(float) * total)) || (rc = ensure(ctx, s->g_u, sizeof(double) * total)) ||
        (rc = ensure(ctx, s->g_dsum, sizeof(float) * std::max(1, n_cols) * total)) ||
        (rc = ensure(ctx, s->g_grad, sizeof(float) * 3 * total)) ||
        (rc = ensure(ctx, s->block_out, sizeof(double) * 4)) ||
        (rc = ensure(ctx, s->g_part, sizeof(double) * n_chunks * (n_cols + 2))) ||
        (rc = ensure(ctx, s->g_cols, sizeof(double) * (n_cols + 2))))
        return rc;
    LaunchArgs a = base_args(s);
    a.sys.charged = 0;
    a.pose_mode = POSE_GRID;
    a.out_mode = OUT_GRID;
    for (int d = 0; d < 3; ++d) a.n_pts[d] = n_pts[d];
    const uint32_t* ax = static_cast<const uint32_t*>(s->axes.p);
    a.grid_x = ax;
    a.grid_y = ax + n_pts[0];
    a.grid_z = ax + n_pts[0] + n_pts[1];
    a.unit_factor = static_cast<float>(unit_factor);
    a.grid_out = static_cast<float*>(s->out_buf.p);
    a.u_out = static_cast<double*>(s->g_u.p);
    a.dsum = static_cast<float*>(s->g_dsum.p);
    a.dsum_stride = total;
    a.grad_u = static_cast<float*>(s->g_grad.p);
    const double inv_t = 1.0 / temperature;
    double* d_scale = static_cast<double*>(s->block_out.p);
    a.grid_bricks = s->cull ? 1 : 0;
    PMGB_CK(ctx, pmgb_launch_pairs_grad(a, s->cull ? pmgb_grid_brick_ctas(n_pts)
                                                   : static_cast<int>((total + PMGB_THREADS - 1) / PMGB_THREADS),
                                        ctx->stream));
    PMGB_CK(ctx, pmgb_launch_max_neg_u(a.u_out, total, inv_t, d_scale, ctx->stream));
    PMGB_CK(ctx, pmgb_launch_weighted_columns(a.u_out, 1, total, inv_t, d_scale, 1, a.dsum, n_cols, total,
                                              static_cast<double*>(s->g_part.p), n_chunks,
                                              static_cast<double*>(s->g_cols.p), ctx->stream));
    // the grid values to the FP64 tolerance (the weights above keep the FP32 energies)
    if (s->exact && (rc = exact_grid(s, n_pts, repfactors, unit_factor, a.grid_out))) return rc;
    std::vector<double> cols(n_cols + 2);
    double M = 0.0;
    PMGB_CK(ctx, cudaMemcpyAsync(out, a.grid_out, sizeof(float) * total, cudaMemcpyDeviceToHost, ctx->stream));
    if (grad_out) PMGB_CK(ctx, cudaMemcpyAsync(grad_out, a.grad_u, sizeof(float) * 3 * total, cudaMemcpyDeviceToHost, ctx->stream));
    PMGB_CK(ctx, cudaMemcpyAsync(cols.data(), s->g_cols.p, sizeof(double) * (n_cols + 2), cudaMemcpyDeviceToHost, ctx->stream));
    PMGB_CK(ctx, cudaMemcpyAsync(&M, d_scale, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if ((rc = check_status(ctx))) return rc;
    dtheta[0] = M;
    dtheta[1] = cols[n_cols];
    dtheta[2] = 0.0;
    assemble_species(s, 1, cols.data(), dtheta);
    return PMGB_OK;
}

extern "C" int pmgb_sample_poses(pmgb_ctx* ctx, uint64_t seed, int64_t start, int64_t n, float* xf_out,
                                 float* rot_out) {
    if (!ctx) return PMGB_ERR_INVALID_ARGUMENT;
    if (n < 0 || start < 0 || (n > 0 && (!xf_out || !rot_out)))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_sample_poses: bad arguments");
    if (n == 0) return PMGB_OK;
    PMGB_CK(ctx, enter_device(ctx->device));
    float *dx = nullptr, *dr = nullptr;
    PMGB_CK(ctx, cudaMalloc(&dx, sizeof(float) * 3 * n));
    cudaError_t e = cudaMalloc(&dr, sizeof(float) * 9 * n);
    if (e == cudaSuccess) e = pmgb_launch_sample_poses(seed, start, n, dx, dr, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(xf_out, dx, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(rot_out, dr, sizeof(float) * 9 * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(dx);
    if (dr) cudaFree(dr);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "pmgb_sample_poses");
    return PMGB_OK;
}

static int grid_axes(pmgb_system* s, const int32_t n_pts[3], const int32_t rep[3]) {
    pmgb_ctx* ctx = s->ctx;
    std::vector<uint32_t> ax;
    std::vector<double> ax64;  // the FP64 fractions, for the double-float re-evaluation
    for (int d = 0; d < 3; ++d)
        for (int i = 0; i < n_pts[d]; ++i) {
            double f = (n_pts[d] > 1) ? static_cast<double>(i) / static_cast<double>(n_pts[d] - 1) : 0.0;
            // the end plane (f = 1) is the periodic image of the first one: evaluate the
            // identical position so both planes hold bit-identical energies
            if (f >= 1.0) f -= 1.0;
            ax.push_back(to_fix(f / rep[d]));
            ax64.push_back(f / rep[d]);
        }
    int rc;
    if ((rc = ensure(ctx, s->axes, sizeof(uint32_t) * ax.size())) || (rc = ensure(ctx, s->axes64, sizeof(double) * ax64.size())))
        return rc;
    if ((rc = staged_h2d(ctx, s->axes.p, ax.data(), sizeof(uint32_t) * ax.size())) ||
        (rc = staged_h2d(ctx, s->axes64.p, ax64.data(), sizeof(double) * ax64.size())))
        return rc;
    return PMGB_OK;
}

// The exact energy grid (grid_axes uploaded): the FP32 pass with each point's rounding-error
// estimate, then the points whose estimate exceeds max(1e-5 |U|, 1e-4 K) re-evaluated in
// double-float (their FP64 energies, rounded to FP32, replace the grid values).
static int exact_grid(pmgb_system* s, const int32_t n_pts[3], const int32_t repfactors[3], double unit_factor,
                      float* out_dev) {
    pmgb_ctx* ctx = s->ctx;
    const int64_t total = int64_t(n_pts[0]) * n_pts[1] * n_pts[2];
    const int n_screen = pmgb_grid_screen_ctas(total);
    int rc;
    if ((rc = ensure(ctx, s->e_bound, sizeof(float) * total)) || (rc = ensure(ctx, s->r_ref, sizeof(double) * 3 * total)))
        return rc;
    LaunchArgs a = base_args(s);
    a.sys.charged = 0;  // grid.jl:337-338: single-site probes get the vdW energy only
    a.pose_mode = POSE_GRID;
    a.out_mode = OUT_GRID;
    for (int d = 0; d < 3; ++d) a.n_pts[d] = n_pts[d];
    const uint32_t* ax = static_cast<const uint32_t*>(s->axes.p);
    a.grid_x = ax;
    a.grid_y = ax + n_pts[0];
    a.grid_z = ax + n_pts[0] + n_pts[1];
    a.unit_factor = static_cast<float>(unit_factor);
    a.grid_out = out_dev;
    a.grid_bricks = 1;
    a.bound_out = static_cast<float*>(s->e_bound.p);
    // worst-case per-term rounding of the FP32 pair terms, and 8 times the rms of independent
    // per-term roundings, both scaled by the box's rounding condition
    a.bound_rho = static_cast<float>(4.0e-6 * s->bound_kappa);
    a.bound_stat = static_cast<float>(4.5e-6 * s->bound_kappa);
    PMGB_CK(ctx, pmgb_launch_grid_bound(a, pmgb_grid_brick_ctas(n_pts), ctx->stream));
    RefineArgs r;
    if ((rc = exact_args(s, total, n_screen, r))) return rc;
    r.sys.charged = 0;
    r.pose_src = REFINE_POSE_GRID;
    for (int d = 0; d < 3; ++d) {
        r.grid_n[d] = n_pts[d];
        r.grid_rep[d] = repfactors[d];
    }
    r.grid_ax64 = static_cast<const double*>(s->axes64.p);
    r.ref_u = static_cast<double*>(s->r_ref.p);
    PMGB_CK(ctx, pmgb_launch_grid_exact(r, a.bound_out, out_dev, total, unit_factor, sm_count(ctx), ctx->stream));
    return PMGB_OK;
}

extern "C" int pmgb_energy_grid_device(pmgb_system* s, const int32_t n_pts[3], const int32_t repfactors[3],
                                       double unit_factor, float* out_dev) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    if (!n_pts || !repfactors || !out_dev)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energy_grid: NULL argument");
    for (int d = 0; d < 3; ++d)
        if (n_pts[d] < 1 || repfactors[d] < 1)
            return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energy_grid: n_pts and repfactors must be >= 1");
    if (s->n_sites != 1)
        return fail(ctx, PMGB_ERR_UNSUPPORTED,
                    "pmgb_energy_grid: the probe must be a single site (got %d sites); multi-site probes need "
                    "rotational averaging",
                    s->n_sites);
    const int64_t total = int64_t(n_pts[0]) * n_pts[1] * n_pts[2];
    if (total > int64_t(INT32_MAX) * PMGB_THREADS / 2)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energy_grid: grid too large");
    if (!(unit_factor > 0.0) || !std::isfinite(unit_factor))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energy_grid: unit_factor must be positive (got %g)",
                    unit_factor);
    PMGB_CK(ctx, enter_device(ctx->device));
    if (int rc = grid_axes(s, n_pts, repfactors)) return rc;
    if (s->exact) return exact_grid(s, n_pts, repfactors, unit_factor, out_dev);
    LaunchArgs a = base_args(s);
    a.sys.charged = 0;  // grid.jl:337-338: single-site probes get the vdW energy only
    a.pose_mode = POSE_GRID;
    a.out_mode = OUT_GRID;
    for (int d = 0; d < 3; ++d) a.n_pts[d] = n_pts[d];
    const uint32_t* ax = static_cast<const uint32_t*>(s->axes.p);
    a.grid_x = ax;
    a.grid_y = ax + n_pts[0];
    a.grid_z = ax + n_pts[0] + n_pts[1];
    a.unit_factor = static_cast<float>(unit_factor);
    a.grid_out = out_dev;
    a.grid_bricks = s->cull ? 1 : 0;  // warps over compact bricks, skipping out-of-cutoff records
    const int n_ctas = s->cull ? pmgb_grid_brick_ctas(n_pts) : static_cast<int>((total + PMGB_THREADS - 1) / PMGB_THREADS);
    PMGB_CK(ctx, pmgb_launch_pairs(a, n_ctas, ctx->stream));
    return PMGB_OK;
}

// The work-counting pass (pmgb_launch_pairs_stats) on prepared arguments; counts_out receives the
// three counters.
static int run_work_counts(pmgb_system* s, LaunchArgs& a, int n_ctas, int64_t counts_out[3], bool img = false) {
    pmgb_ctx* ctx = s->ctx;
    if (int rc = ensure(ctx, s->stats, sizeof(unsigned long long) * 3)) return rc;
    a.stats = static_cast<unsigned long long*>(s->stats.p);
    PMGB_CK(ctx, cudaMemsetAsync(a.stats, 0, sizeof(unsigned long long) * 3, ctx->stream));
    const cudaError_t e = img ? pmgb_launch_pairs_img(a, n_ctas, ctx->stream) : pmgb_launch_pairs_stats(a, n_ctas, ctx->stream);
    if (e == cudaErrorNotSupported)
        return fail(ctx, PMGB_ERR_UNSUPPORTED, "work counts: guests of one or three sites only (got %d)", s->n_sites);
    PMGB_CK(ctx, e);
    unsigned long long c[3] = {0, 0, 0};
    PMGB_CK(ctx, cudaMemcpyAsync(c, a.stats, sizeof(c), cudaMemcpyDeviceToHost, ctx->stream));
    if (int rc = check_status(ctx)) return rc;
    for (int i = 0; i < 3; ++i) counts_out[i] = static_cast<int64_t>(c[i]);
    return PMGB_OK;
}

extern "C" int pmgb_widom_work_counts(pmgb_system* s, int64_t n_per_block, int32_t n_blocks, uint64_t seed,
                                      int64_t counts_out[3]) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    if (n_per_block < 1 || n_blocks < 1 || !counts_out)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom_work_counts: bad arguments");
    if (int rc = ready_for_charges(s)) return rc;
    if (n_per_block > static_cast<int64_t>(INT32_MAX) * PMGB_THREADS)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom_work_counts: too many insertions per block");
    const int64_t cpb = (n_per_block + PMGB_THREADS - 1) / PMGB_THREADS;
    if (cpb > INT32_MAX / n_blocks) return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom_work_counts: too many");
    PMGB_CK(ctx, enter_device(ctx->device));
    const size_t n_ins = static_cast<size_t>(n_per_block) * n_blocks;
    const bool img = uses_image_lists(s, static_cast<int64_t>(n_ins));
    if (img && n_ins > static_cast<size_t>(INT32_MAX))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_widom_work_counts: too many insertions for one run");
    const size_t n_cells = img ? size_t{1} << (3 * pmgb_run_order_bits(static_cast<long long>(n_ins)))
                               : pmgb_widom_order_cells() * n_blocks;
    int rc;
    if ((rc = ensure(ctx, s->o_counts, sizeof(int) * n_cells)) || (rc = ensure(ctx, s->o_perm, sizeof(int) * n_ins)))
        return rc;
    LaunchArgs a = base_args(s);
    a.pose_mode = POSE_PHILOX;
    a.out_mode = OUT_WIDOM;
    a.seed = seed;
    a.n_per_block = n_per_block;
    a.n_blocks = n_blocks;
    a.ctas_per_block = static_cast<int>(cpb);
    a.inv_temperature = 1.0;
    a.perm = static_cast<const int*>(s->o_perm.p);  // the spatially ordered pass of pmgb_widom_device
    if (img) {
        if ((rc = ensure(ctx, s->g_u, sizeof(double) * 2 * n_ins))) return rc;
        a.u_out = static_cast<double*>(s->g_u.p);
        PMGB_CK(ctx, pmgb_launch_run_order(seed, static_cast<long long>(n_ins), static_cast<int*>(s->o_counts.p),
                                           static_cast<int*>(s->o_perm.p), ctx->stream));
        return run_work_counts(s, a, static_cast<int>(cpb * n_blocks), counts_out, true);
    }
    PMGB_CK(ctx, pmgb_launch_widom_order(seed, n_per_block, n_blocks, static_cast<int*>(s->o_counts.p),
                                         static_cast<int*>(s->o_perm.p), ctx->stream));
    return run_work_counts(s, a, static_cast<int>(cpb * n_blocks), counts_out);
}

extern "C" int pmgb_energy_grid_work_counts(pmgb_system* s, const int32_t n_pts[3], const int32_t repfactors[3],
                                            int64_t counts_out[3]) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    if (!n_pts || !repfactors || !counts_out)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energy_grid_work_counts: NULL argument");
    for (int d = 0; d < 3; ++d)
        if (n_pts[d] < 1 || repfactors[d] < 1)
            return fail(ctx, PMGB_ERR_INVALID_ARGUMENT,
                        "pmgb_energy_grid_work_counts: n_pts and repfactors must be >= 1");
    if (s->n_sites != 1)
        return fail(ctx, PMGB_ERR_UNSUPPORTED, "pmgb_energy_grid_work_counts: the probe must be a single site");
    const int64_t total = int64_t(n_pts[0]) * n_pts[1] * n_pts[2];
    if (total > int64_t(INT32_MAX) * PMGB_THREADS / 2)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energy_grid_work_counts: grid too large");
    PMGB_CK(ctx, enter_device(ctx->device));
    if (int rc = grid_axes(s, n_pts, repfactors)) return rc;
    if (int rc = ensure(ctx, s->out_buf, sizeof(float) * total)) return rc;
    LaunchArgs a = base_args(s);
    a.sys.charged = 0;  // grid.jl:337-338: single-site probes get the vdW energy only
    a.pose_mode = POSE_GRID;
    a.out_mode = OUT_GRID;
    for (int d = 0; d < 3; ++d) a.n_pts[d] = n_pts[d];
    const uint32_t* ax = static_cast<const uint32_t*>(s->axes.p);
    a.grid_x = ax;
    a.grid_y = ax + n_pts[0];
    a.grid_z = ax + n_pts[0] + n_pts[1];
    a.unit_factor = 1.0f;
    a.grid_out = static_cast<float*>(s->out_buf.p);
    a.grid_bricks = 1;  // the brick order of the grid pass
    return run_work_counts(s, a, pmgb_grid_brick_ctas(n_pts), counts_out);
}

extern "C" int pmgb_energy_grid_rotational(pmgb_system* s, const int32_t n_pts[3], const int32_t repfactors[3],
                                           int32_t n_rotations, double temperature, uint64_t seed, double unit_factor,
                                           float* out) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    if (!n_pts || !repfactors || !out)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energy_grid_rotational: NULL argument");
    for (int d = 0; d < 3; ++d)
        if (n_pts[d] < 1 || repfactors[d] < 1)
            return fail(ctx, PMGB_ERR_INVALID_ARGUMENT,
                        "pmgb_energy_grid_rotational: n_pts and repfactors must be >= 1");
    if (n_rotations < 1)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energy_grid_rotational: n_rotations must be >= 1");
    if (!(temperature > 0.0) || !std::isfinite(temperature))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT,
                    "pmgb_energy_grid_rotational: Must pass temperature (K) for Boltzmann weighted rotations "
                    "(got %g)", temperature);
    if (!(unit_factor > 0.0) || !std::isfinite(unit_factor))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energy_grid_rotational: unit_factor must be positive");
    if (int rc = ready_for_charges(s)) return rc;
    const int64_t total = int64_t(n_pts[0]) * n_pts[1] * n_pts[2];
    if (total > INT32_MAX) return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energy_grid_rotational: grid too large");
    PMGB_CK(ctx, enter_device(ctx->device));
    if (int rc = grid_axes(s, n_pts, repfactors)) return rc;
    // the points in slices of at most ~8M insertions, bounding the per-insertion scratch
    const int64_t cpb = (int64_t(n_rotations) + PMGB_THREADS - 1) / PMGB_THREADS;
    const int64_t slice = std::max<int64_t>(1, std::min<int64_t>(total, (int64_t(1) << 23) / n_rotations));
    const bool refine = s->exact || s->refine_tail > 0.0;
    const double tail = s->refine_tail > 0.0 ? s->refine_tail : 1e-3;
    int rc;
    if ((rc = ensure(ctx, s->out_buf, sizeof(float) * total)) ||
        (rc = ensure(ctx, s->partials, sizeof(LsePartial) * slice * cpb)) ||
        (rc = ensure(ctx, s->block_out, sizeof(double) * 4 * slice)) ||
        (refine && (rc = ensure(ctx, s->g_u, sizeof(double) * 2 * slice * n_rotations))))
        return rc;
    const uint32_t* ax = static_cast<const uint32_t*>(s->axes.p);
    for (int64_t p0 = 0; p0 < total; p0 += slice) {
        const int nb = static_cast<int>(std::min(slice, total - p0));
        LaunchArgs a = base_args(s);
        a.pose_mode = POSE_PHILOX;
        a.out_mode = OUT_WIDOM;
        a.seed = seed;
        a.n_per_block = n_rotations;
        a.n_blocks = nb;
        a.ctas_per_block = static_cast<int>(cpb);
        a.inv_temperature = 1.0 / temperature;
        a.partials = static_cast<LsePartial*>(s->partials.p);
        a.u_out = refine ? static_cast<double*>(s->g_u.p) : nullptr;
        a.no_resid = refine ? 1 : 0;
        a.rot_grid = 1;
        a.point_base = p0;
        a.item_base = p0 * n_rotations;
        for (int d = 0; d < 3; ++d) a.n_pts[d] = n_pts[d];
        a.grid_x = ax;
        a.grid_y = ax + n_pts[0];
        a.grid_z = ax + n_pts[0] + n_pts[1];
        double* bo = static_cast<double*>(s->block_out.p);
        PMGB_CK(ctx, pmgb_launch_pairs(a, static_cast<int>(nb * cpb), ctx->stream));
        PMGB_CK(ctx, pmgb_launch_reduce_blocks(a.partials, nb, a.ctas_per_block, bo, ctx->stream));
        if (refine) {
            RefineArgs where{};
            for (int d = 0; d < 3; ++d) {
                where.grid_n[d] = n_pts[d];
                where.grid_rep[d] = repfactors[d];
            }
            where.grid_ax64 = static_cast<const double*>(s->axes64.p);
            where.point_base = p0;
            where.item_base = a.item_base;
            if ((rc = run_refine(s, n_rotations, nb, seed, temperature, bo, a.u_out, tail, &where))) return rc;
        }
        PMGB_CK(ctx, pmgb_launch_rot_grid_out(bo, nb, temperature, std::log(static_cast<double>(n_rotations)),
                                              unit_factor, static_cast<float*>(s->out_buf.p) + p0, ctx->stream));
    }
    PMGB_CK(ctx, cudaMemcpyAsync(out, s->out_buf.p, sizeof(float) * total, cudaMemcpyDeviceToHost, ctx->stream));
    return check_status(ctx);
}

extern "C" int pmgb_energy_grid(pmgb_system* s, const int32_t n_pts[3], const int32_t repfactors[3],
                                double unit_factor, float* out) {
    if (!s) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = s->ctx;
    if (!out || !n_pts) return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_energy_grid: NULL argument");
    PMGB_CK(ctx, enter_device(ctx->device));
    const int64_t total = int64_t(std::max(n_pts[0], 0)) * std::max(n_pts[1], 0) * std::max(n_pts[2], 0);
    if (int rc = ensure(ctx, s->out_buf, sizeof(float) * std::max<int64_t>(total, 1))) return rc;
    if (int rc = pmgb_energy_grid_device(s, n_pts, repfactors, unit_factor, static_cast<float*>(s->out_buf.p)))
        return rc;
    PMGB_CK(ctx, cudaMemcpyAsync(out, s->out_buf.p, sizeof(float) * total, cudaMemcpyDeviceToHost, ctx->stream));
    return check_status(ctx);
}

extern "C" int pmgb_philox4x32_10(pmgb_ctx* ctx, int64_t n, const uint32_t* ctr, const uint32_t* key,
                                  uint32_t* out) {
    if (!ctx) return PMGB_ERR_INVALID_ARGUMENT;
    if (n < 0 || (n > 0 && (!ctr || !key || !out)))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_philox4x32_10: bad arguments");
    if (n == 0) return PMGB_OK;
    PMGB_CK(ctx, enter_device(ctx->device));
    unsigned int *dc = nullptr, *dk = nullptr, *dout = nullptr;
    cudaError_t e = cudaMalloc(&dc, 16 * n);
    if (e == cudaSuccess) e = cudaMalloc(&dk, 8 * n);
    if (e == cudaSuccess) e = cudaMalloc(&dout, 16 * n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dc, ctr, 16 * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dk, key, 8 * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = pmgb_launch_philox(dc, dk, n, dout, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, 16 * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (dc) cudaFree(dc);
    if (dk) cudaFree(dk);
    if (dout) cudaFree(dout);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "pmgb_philox4x32_10");
    return PMGB_OK;
}

extern "C" int pmgb_vdw_energy_ordered(pmgb_ctx* ctx, const double f_to_c[9], int32_t n_atoms, const double* atom_xf,
                                       const int32_t* atom_species, int32_t n_species, const double* eps,
                                       const double* sigma2, double r2_cutoff, int64_t n_conf, int32_t n_sites,
                                       const int32_t* site_species, const double* site_xf, double* out) {
    if (!ctx) return PMGB_ERR_INVALID_ARGUMENT;
    if (!f_to_c || n_atoms < 0 || (n_atoms > 0 && (!atom_xf || !atom_species)) || n_species < 1 || !eps ||
        !sigma2 || n_conf < 0 || n_sites < 1 || !site_species || (n_conf > 0 && (!site_xf || !out)) ||
        n_conf > (int64_t{1} << 40) / n_sites)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_vdw_energy_ordered: bad arguments");
    for (int32_t j = 0; j < n_atoms; ++j)
        if (atom_species[j] < 0 || atom_species[j] >= n_species)
            return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_vdw_energy_ordered: atom species out of range");
    for (int32_t i = 0; i < n_sites; ++i)
        if (site_species[i] < 0 || site_species[i] >= n_species)
            return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_vdw_energy_ordered: site species out of range");
    if (n_conf == 0) return PMGB_OK;
    PMGB_CK(ctx, enter_device(ctx->device));
    const size_t nt = static_cast<size_t>(n_species) * n_species;
    const size_t b_f = 9 * sizeof(double), b_ax = 3 * sizeof(double) * n_atoms, b_as = sizeof(int) * n_atoms,
                 b_t = sizeof(double) * nt, b_ss = sizeof(int) * n_sites,
                 b_sx = 3 * sizeof(double) * static_cast<size_t>(n_conf) * n_sites, b_o = sizeof(double) * n_conf;
    // one allocation, each part on a 256-byte boundary
    auto up = [](size_t b) { return (b + 255) & ~size_t{255}; };
    const size_t o_ax = up(b_f), o_as = o_ax + up(b_ax), o_e = o_as + up(b_as), o_s = o_e + up(b_t),
                 o_ss = o_s + up(b_t), o_sx = o_ss + up(b_ss), o_o = o_sx + up(b_sx), total = o_o + up(b_o);
    char* d = nullptr;
    cudaError_t e = cudaMalloc(&d, total);
    auto h2d = [&](size_t off, const void* src, size_t b) {
        if (e == cudaSuccess && b) e = cudaMemcpyAsync(d + off, src, b, cudaMemcpyHostToDevice, ctx->stream);
    };
    h2d(0, f_to_c, b_f);
    h2d(o_ax, atom_xf, b_ax);
    h2d(o_as, atom_species, b_as);
    h2d(o_e, eps, b_t);
    h2d(o_s, sigma2, b_t);
    h2d(o_ss, site_species, b_ss);
    h2d(o_sx, site_xf, b_sx);
    if (e == cudaSuccess)
        e = pmgb_launch_vdw_ordered(reinterpret_cast<const double*>(d), n_atoms,
                                    reinterpret_cast<const double*>(d + o_ax), reinterpret_cast<const int*>(d + o_as),
                                    n_species, reinterpret_cast<const double*>(d + o_e),
                                    reinterpret_cast<const double*>(d + o_s), r2_cutoff, n_conf, n_sites,
                                    reinterpret_cast<const int*>(d + o_ss), reinterpret_cast<const double*>(d + o_sx),
                                    reinterpret_cast<double*>(d + o_o), ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d + o_o, b_o, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (d) cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "pmgb_vdw_energy_ordered");
    return PMGB_OK;
}

extern "C" int pmgb_fp32_peak(pmgb_ctx* ctx, int n_ctas, int iters, double* tflops_out) {
    if (!ctx || !tflops_out || n_ctas < 1 || iters < 1) return PMGB_ERR_INVALID_ARGUMENT;
    PMGB_CK(ctx, enter_device(ctx->device));
    float* sink = nullptr;
    PMGB_CK(ctx, cudaMalloc(&sink, sizeof(float) * n_ctas));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaError_t e = pmgb_launch_fp32_peak(sink, n_ctas, iters, ctx->stream);  // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(e0, ctx->stream);
    if (e == cudaSuccess) e = pmgb_launch_fp32_peak(sink, n_ctas, iters, ctx->stream);
    if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "pmgb_fp32_peak");
    const double flops = 2.0 * 8.0 * 16.0 * double(iters) * 256.0 * double(n_ctas);
    *tflops_out = flops / (double(ms) * 1e-3) / 1e12;
    return PMGB_OK;
}

// ============================================================================
// batched screening
// ============================================================================
struct pmgb_batch {
    pmgb_ctx* ctx = nullptr;
    std::vector<pmgb_system*> systems;
    std::vector<BatchSystem> host_sys;
    std::vector<double> chunk_flops;   // per system: algorithmic flops of one chunk
    std::vector<BatchUnit> units;      // current work units
    std::vector<double> unit_cost;
    int n_blocks = 0;
    bool grad = false;
    int n_ctas = 0, order = 0, max_ctas = 0, sm_count = 0, max_cols = 0;
    double unit_mflop = 0.0;           // target work per unit (0: one chunk per unit)
    int64_t n_chunks = 0, n_out_cols = 0, n_insertions = 0, dtheta_len = 0, device_bytes = 0;
    // device memory
    BatchSystem* d_sys = nullptr;
    BatchUnit* d_units = nullptr;
    int* d_order = nullptr;
    int* d_counter = nullptr;
    BatchRun* d_run = nullptr;
    LsePartial* d_partials = nullptr;
    float* d_dsum = nullptr;
    double* d_unit_cols = nullptr;
    double* d_block_out = nullptr;
    double* d_out_cols = nullptr;
    // FP64 tail refinement (off when refine_tail == 0)
    double refine_tail = 0.0;
    int* d_chunk_sys = nullptr;
    double* d_u = nullptr;
    unsigned long long* d_hist = nullptr;
    int *d_cut = nullptr, *d_counts = nullptr, *d_offsets = nullptr;
    long long* d_list = nullptr;
    double* d_ref_u = nullptr;
    int *d_plan = nullptr, *d_done = nullptr;
    double* d_part = nullptr;
    // spatial order with cutoff culling (off: insertions in index order)
    bool cull = false;
    int* d_perm = nullptr;
    int* d_cells = nullptr;
    double* d_unit_m = nullptr;
    // image-list systems (forward runs with refinement): one order over each system's run
    int64_t img_cells = 0;             // sum over systems of 2^(3 order_bits)
    int* d_img_cells = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool launched = false;
};

namespace {

void batch_free(pmgb_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    void* ptrs[] = {b->d_sys, b->d_units, b->d_order, b->d_counter, b->d_run, b->d_partials,
                    b->d_dsum, b->d_unit_cols, b->d_block_out, b->d_out_cols, b->d_chunk_sys, b->d_u,
                    b->d_hist, b->d_cut, b->d_counts, b->d_offsets, b->d_list, b->d_ref_u,
                    b->d_plan, b->d_done, b->d_part, b->d_perm, b->d_cells, b->d_unit_m, b->d_img_cells};
    for (void* p : ptrs) dev_free(b->ctx, p);
}

template <class T>
int batch_alloc(pmgb_batch* b, T** p, size_t count) {
    const size_t bytes = std::max<size_t>(count * sizeof(T), 16);
    PMGB_CK(b->ctx, dev_malloc(b->ctx, reinterpret_cast<void**>(p), bytes));
    b->device_bytes += static_cast<int64_t>(bytes);
    return PMGB_OK;
}

// Capture memset(counter) + persistent kernel + per-system reduction as one graph.
int batch_capture(pmgb_batch* b) {
    pmgb_ctx* ctx = b->ctx;
    if (b->exec) {
        PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    // image lists for the systems that allow them, in runs with spatial order (the adjoint's
    // columns formed in the list loop)
    bool any_img = false, changed = false;
    for (size_t i = 0; i < b->systems.size(); ++i) {
        const int img = (b->cull &&
                         image_lists_for(b->systems[i], b->host_sys[i].n_per_block * b->n_blocks, true)) ? 1 : 0;
        changed = changed || b->host_sys[i].img != img;
        b->host_sys[i].img = img;
        any_img = any_img || img;
    }
    if (any_img && !b->d_img_cells)
        if (int rc = batch_alloc(b, &b->d_img_cells, static_cast<size_t>(b->img_cells))) return rc;
    if (changed) {
        PMGB_CK(ctx, cudaMemcpyAsync(b->d_sys, b->host_sys.data(), sizeof(BatchSystem) * b->host_sys.size(),
                                     cudaMemcpyHostToDevice, ctx->stream));
        PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));  // host_sys may change again before the next upload
    }
    BatchArgs a{};
    a.systems = b->d_sys;
    a.units = b->d_units;
    a.order = b->d_order;
    a.n_units = static_cast<int>(b->units.size());
    a.counter = b->d_counter;
    a.run = b->d_run;
    a.partials = b->d_partials;
    a.status = ctx->d_status;
    a.dsum = b->d_dsum;
    a.max_cols = b->max_cols;
    a.unit_cols = b->d_unit_cols;
    a.u = (b->refine_tail > 0.0 || b->cull) ? b->d_u : nullptr;
    a.perm = b->cull ? b->d_perm : nullptr;
    a.unit_m = b->cull ? b->d_unit_m : nullptr;
    a.no_resid = (b->refine_tail > 0.0 && !b->grad) ? 1 : 0;
    RefineArgs r{};
    if (b->refine_tail > 0.0) {
        r.systems = b->d_sys;
        r.chunk_sys = b->d_chunk_sys;
        r.run = b->d_run;
        r.n_systems = static_cast<int>(b->systems.size());
        r.n_blocks = b->n_blocks;
        r.tail = b->refine_tail;
        r.block_out = b->d_block_out;
        r.partials = b->d_partials;
        r.u = b->d_u;
        r.hist = b->d_hist;
        r.cut = b->d_cut;
        r.counts = b->d_counts;
        r.offsets = b->d_offsets;
        r.list = b->d_list;
        r.ref_u = b->d_ref_u;
        r.counter = b->d_offsets + b->n_chunks + 1;
        r.plan = b->d_plan;
        r.one_chunk = b->d_plan + b->systems.size() + 1;
        r.done = b->d_done;
        r.part = b->d_part;
        r.cap_entries = b->n_insertions;
        r.cap_items = 2 * b->n_insertions + 4096;
    }
    cudaStream_t st = ctx->stream;
    PMGB_CK(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int n_sys = static_cast<int>(b->systems.size()), n_chunks = static_cast<int>(b->n_chunks);
    cudaError_t e = cudaMemsetAsync(b->d_counter, 0, sizeof(int), st);
    if (e == cudaSuccess && b->cull)
        e = pmgb_launch_batch_order(b->d_sys, b->d_chunk_sys, n_chunks, n_sys, b->n_blocks, b->d_run, b->d_cells,
                                    b->d_perm, st);
    if (e == cudaSuccess && any_img)
        e = pmgb_launch_batch_run_order(b->d_sys, b->d_chunk_sys, n_chunks, n_sys, b->d_run, b->d_img_cells,
                                        b->img_cells, b->d_perm, st);
    if (e == cudaSuccess) e = pmgb_launch_batch(a, b->grad, b->n_ctas, st);
    if (e == cudaSuccess && b->cull)
        e = pmgb_launch_batch_lse(b->d_sys, b->d_chunk_sys, n_chunks, b->d_run, b->d_u, b->d_partials, st);
    if (e == cudaSuccess)
        e = pmgb_launch_batch_reduce(b->d_sys, n_sys, b->n_blocks, b->d_partials, b->d_unit_cols, a.unit_m, b->grad,
                                     b->d_block_out, b->d_out_cols, st);
    if (e == cudaSuccess && b->refine_tail > 0.0)
        e = pmgb_launch_refine(r, static_cast<int>(b->n_chunks), b->sm_count, st);
    cudaGraph_t g = nullptr;
    const cudaError_t e_end = cudaStreamEndCapture(st, &g);
    if (e == cudaSuccess) e = e_end;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "pmgb_batch: graph capture");
    return PMGB_OK;
}

// Cut every system's chunks into work units of about unit_mflop of work (whole blocks at
// most; one chunk per unit for frameworks that do not fit the ring) and upload them with
// their processing order: 0 = estimated cost, largest first; 1 = system by system.
int batch_build_units(pmgb_batch* b, double unit_mflop, int order) {
    b->units.clear();
    b->unit_cost.clear();
    for (size_t i = 0; i < b->host_sys.size(); ++i) {
        const BatchSystem& bs = b->host_sys[i];
        const int cpb = bs.ctas_per_block;
        int g = 1;
        if (unit_mflop > 0.0 && bs.sys.n_tiles <= PMGB_NSTAGE)
            g = static_cast<int>(std::min<double>(cpb, std::max(1.0, std::ceil(unit_mflop * 1e6 / b->chunk_flops[i]))));
        for (int blk = 0; blk < b->n_blocks; ++blk)
            for (int c0 = 0; c0 < cpb; c0 += g) {
                const int n = std::min(g, cpb - c0);
                b->units.push_back(BatchUnit{static_cast<int>(i), blk, c0, n});
                b->unit_cost.push_back(n * b->chunk_flops[i]);
            }
    }
    const int n = static_cast<int>(b->units.size());
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    if (order == 0)
        std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return b->unit_cost[x] > b->unit_cost[y]; });
    pmgb_ctx* ctx = b->ctx;
    PMGB_CK(ctx, cudaMemcpyAsync(b->d_units, b->units.data(), sizeof(BatchUnit) * n, cudaMemcpyHostToDevice,
                                 ctx->stream));
    PMGB_CK(ctx, cudaMemcpyAsync(b->d_order, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));  // idx is a local
    b->order = order;
    b->unit_mflop = unit_mflop;
    return PMGB_OK;
}

// Per-insertion energies and the chunk -> system map, shared by the refinement and the
// spatial order; allocated on first use.
int batch_ensure_u(pmgb_batch* b) {
    if (b->d_u) return PMGB_OK;
    pmgb_ctx* ctx = b->ctx;
    std::vector<int> chunk_sys(static_cast<size_t>(b->n_chunks));
    for (size_t i = 0; i < b->host_sys.size(); ++i) {
        const BatchSystem& bs = b->host_sys[i];
        const int64_t n_c = static_cast<int64_t>(bs.ctas_per_block) * b->n_blocks;
        for (int64_t c = 0; c < n_c; ++c) chunk_sys[bs.chunk_first + c] = static_cast<int>(i);
    }
    int rc;
    if ((rc = batch_alloc(b, &b->d_chunk_sys, chunk_sys.size())) ||
        (rc = batch_alloc(b, &b->d_u, 2 * static_cast<size_t>(b->n_insertions))))
        return rc;
    PMGB_CK(ctx, cudaMemcpyAsync(b->d_chunk_sys, chunk_sys.data(), sizeof(int) * chunk_sys.size(),
                                 cudaMemcpyHostToDevice, ctx->stream));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));  // chunk_sys is a local
    return PMGB_OK;
}

int batch_enqueue(pmgb_batch* b, uint64_t seed, double temperature) {
    pmgb_ctx* ctx = b->ctx;
    const BatchRun run{static_cast<unsigned long long>(seed), 1.0 / temperature};
    // pageable source: staged at once, so the local may go out of scope
    PMGB_CK(ctx, cudaMemcpyAsync(b->d_run, &run, sizeof(run), cudaMemcpyHostToDevice, ctx->stream));
    PMGB_CK(ctx, cudaGraphLaunch(b->exec, ctx->stream));
    b->launched = true;
    return PMGB_OK;
}

}  // namespace

extern "C" int pmgb_batch_create(pmgb_ctx* ctx, int32_t n_systems, pmgb_system* const* systems,
                                 const int64_t* n_per_block, int32_t n_blocks, int32_t with_adjoint,
                                 pmgb_batch** out) {
    if (!ctx) return PMGB_ERR_INVALID_ARGUMENT;
    if (!out || n_systems < 1 || !systems || !n_per_block || n_blocks < 1)
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_batch_create: bad arguments");
    *out = nullptr;
    PMGB_CK(ctx, enter_device(ctx->device));
    auto* b = new pmgb_batch();
    b->ctx = ctx;
    b->n_blocks = n_blocks;
    b->grad = with_adjoint != 0;
    int64_t col_base = 0, out_base = 0, n_chunks = 0;
    for (int32_t i = 0; i < n_systems; ++i) {
        pmgb_system* s = systems[i];
        const char* why = nullptr;
        if (!s) why = "NULL system";
        else if (s->ctx != ctx) why = "system belongs to another context";
        else if (s->dev.charged && !s->ewald_set) why = "charged system without pmgb_system_set_ewald";
        else if (n_per_block[i] < 1) why = "n_per_block < 1";
        if (why) {
            delete b;
            return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_batch_create: system %d: %s", i, why);
        }
        const int variant = pmgb_batch_variant(s->n_sites, s->dev.charged != 0);
        if (variant < 0) {
            delete b;
            return fail(ctx, PMGB_ERR_UNSUPPORTED, "pmgb_batch_create: system %d: %d guest sites", i, s->n_sites);
        }
        const int64_t cpb = (n_per_block[i] + PMGB_THREADS - 1) / PMGB_THREADS;
        const int nst = template_sites(s->n_sites);
        BatchSystem bs{};
        bs.sys = s->dev;
        bs.n_per_block = n_per_block[i];
        bs.variant = variant;
        bs.n_cols = b->grad ? s->dev.n_seg * nst * 2 : 0;
        bs.chunk_first = static_cast<int>(n_chunks);
        bs.ctas_per_block = static_cast<int>(cpb);
        bs.col_base = col_base;
        bs.out_base = out_base;
        bs.u_base = b->n_insertions;
        bs.img = 0;  // set with the run's settings (batch_capture)
        bs.order_bits = pmgb_run_order_bits(n_per_block[i] * n_blocks);
        bs.cell_base = b->img_cells;
        b->img_cells += int64_t{1} << (3 * bs.order_bits);
        // cost model of one chunk: algorithmic flops of its pair and reciprocal-space terms
        const double pair = s->dev.charged ? 68.0 : 28.0;
        b->chunk_flops.push_back(PMGB_THREADS * nst *
                                 (pair * s->dev.n_rec + (s->dev.charged ? 17.0 * s->dev.n_k : 0.0)) + 1.0);
        n_chunks += cpb * n_blocks;
        if (n_chunks > INT32_MAX / 2) {
            delete b;
            return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_batch_create: too many insertions");
        }
        col_base += cpb * n_blocks * bs.n_cols;
        out_base += 3 + bs.n_cols;
        b->max_cols = std::max(b->max_cols, bs.n_cols);
        b->n_insertions += n_per_block[i] * n_blocks;
        b->dtheta_len += 3 + 2 * static_cast<int64_t>(s->n_species) * s->n_species;
        b->host_sys.push_back(bs);
        b->systems.push_back(s);
    }
    b->n_chunks = n_chunks;
    b->n_out_cols = out_base;
    cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, ctx->device);
    int rc = PMGB_OK;
    cudaError_t e = pmgb_batch_prepare(b->grad);
    if (e != cudaSuccess) rc = cuda_fail(ctx, e, "pmgb_batch_create: kernel attributes");
    b->max_ctas = std::max(1, 2 * b->sm_count);
    b->n_ctas = b->max_ctas;
    if (!rc) rc = batch_alloc(b, &b->d_sys, b->host_sys.size());
    if (!rc) rc = batch_alloc(b, &b->d_units, static_cast<size_t>(n_chunks));  // one chunk per unit at most
    if (!rc) rc = batch_alloc(b, &b->d_order, static_cast<size_t>(n_chunks));
    if (!rc) rc = batch_alloc(b, &b->d_counter, 1);
    if (!rc) rc = batch_alloc(b, &b->d_run, 1);
    if (!rc) rc = batch_alloc(b, &b->d_partials, static_cast<size_t>(n_chunks));
    if (!rc) rc = batch_alloc(b, &b->d_block_out, b->host_sys.size() * 4 * n_blocks);
    if (!rc && b->grad) rc = batch_alloc(b, &b->d_dsum, static_cast<size_t>(b->max_ctas) * b->max_cols * PMGB_THREADS);
    if (!rc && b->grad) rc = batch_alloc(b, &b->d_unit_cols, static_cast<size_t>(col_base));
    if (!rc && b->grad) rc = batch_alloc(b, &b->d_out_cols, static_cast<size_t>(out_base));
    if (!rc) {
        e = cudaMemcpyAsync(b->d_sys, b->host_sys.data(), sizeof(BatchSystem) * b->host_sys.size(),
                            cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) rc = cuda_fail(ctx, e, "pmgb_batch_create: upload");
    }
    if (!rc) rc = batch_build_units(b, 0.0, 0);  // synchronises: the upload above reads host_sys
    if (!rc) rc = pmgb_batch_set_cull(b, 1);      // on by default, as for a system; captures the graph
    if (rc) {
        batch_free(b);
        delete b;
        return rc;
    }
    ++ctx->refs;
    for (pmgb_system* sy : b->systems) ++sy->refs;  // the batch reads them: keep them alive with it
    *out = b;
    return PMGB_OK;
}

extern "C" void pmgb_batch_destroy(pmgb_batch* b) {
    if (!b) return;
    pmgb_ctx* ctx = b->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    batch_free(b);
    for (pmgb_system* sy : b->systems) system_release(sy);
    delete b;
    ctx_release(ctx);
    (void)cudaGetLastError();
}

extern "C" int pmgb_batch_configure(pmgb_batch* b, int32_t n_ctas, int32_t order, double unit_mflop) {
    if (!b) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = b->ctx;
    if (n_ctas < 0 || n_ctas > b->max_ctas || (order != 0 && order != 1) || !(unit_mflop >= 0.0))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT,
                    "pmgb_batch_configure: n_ctas in [0, %d], order 0 or 1, unit_mflop >= 0", b->max_ctas);
    PMGB_CK(ctx, enter_device(ctx->device));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    b->n_ctas = n_ctas == 0 ? b->max_ctas : n_ctas;
    if (int rc = batch_build_units(b, unit_mflop, order)) return rc;
    b->launched = false;
    return batch_capture(b);
}

extern "C" int pmgb_batch_set_refine(pmgb_batch* b, double tail_fraction) {
    if (!b) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = b->ctx;
    if (!(tail_fraction >= 0.0 && tail_fraction < 1.0))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_batch_set_refine: tail fraction in [0, 1)");
    PMGB_CK(ctx, enter_device(ctx->device));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (tail_fraction > 0.0 && !b->d_hist) {
        // scratch sized for the worst case: every insertion refined
        const size_t n = static_cast<size_t>(b->n_insertions), g = b->systems.size() * b->n_blocks;
        const size_t n_chunks = static_cast<size_t>(b->n_chunks);
        int rc;
        if ((rc = batch_ensure_u(b)) || (rc = batch_alloc(b, &b->d_hist, g * pmgb_refine_hist_words())) ||
            (rc = batch_alloc(b, &b->d_cut, g)) || (rc = batch_alloc(b, &b->d_counts, n_chunks)) ||
            (rc = batch_alloc(b, &b->d_offsets, n_chunks + 2)) || (rc = batch_alloc(b, &b->d_list, n)) ||
            (rc = batch_alloc(b, &b->d_ref_u, 3 * n)) || (rc = batch_alloc(b, &b->d_plan, b->systems.size() + 2)) ||
            (rc = batch_alloc(b, &b->d_done, n)) || (rc = batch_alloc(b, &b->d_part, 4 * (2 * n + 4096))))
            return rc;
    }
    b->refine_tail = tail_fraction;
    b->launched = false;
    return batch_capture(b);
}

extern "C" int pmgb_batch_set_cull(pmgb_batch* b, int32_t on) {
    if (!b) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = b->ctx;
    PMGB_CK(ctx, enter_device(ctx->device));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (on && !b->d_perm) {
        const size_t cells = b->systems.size() * b->n_blocks * pmgb_batch_order_cells();
        int rc;
        if ((rc = batch_ensure_u(b)) || (rc = batch_alloc(b, &b->d_perm, static_cast<size_t>(b->n_insertions))) ||
            (rc = batch_alloc(b, &b->d_cells, cells)) ||
            (b->grad && (rc = batch_alloc(b, &b->d_unit_m, static_cast<size_t>(b->n_chunks)))))
            return rc;
    }
    b->cull = on != 0;
    b->launched = false;
    return batch_capture(b);
}

extern "C" int pmgb_batch_launch(pmgb_batch* b, uint64_t seed, double temperature) {
    if (!b) return PMGB_ERR_INVALID_ARGUMENT;
    if (!(temperature > 0.0) || !std::isfinite(temperature))
        return fail(b->ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_batch_launch: temperature must be positive");
    PMGB_CK(b->ctx, enter_device(b->ctx->device));
    return batch_enqueue(b, seed, temperature);
}

extern "C" int pmgb_batch_tune(pmgb_batch* b, uint64_t seed, double temperature, int32_t repeats,
                               double* best_ms_out) {
    if (!b) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = b->ctx;
    if (repeats < 1 || !(temperature > 0.0))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_batch_tune: repeats >= 1 and a positive temperature");
    PMGB_CK(ctx, enter_device(ctx->device));
    cudaEvent_t e0, e1;
    PMGB_CK(ctx, cudaEventCreate(&e0));
    PMGB_CK(ctx, cudaEventCreate(&e1));
    struct Shape {
        int n_ctas, order;
        double mflop;
    };
    double best = INFINITY;
    Shape best_s{b->max_ctas, 0, 0.0};
    int rc = PMGB_OK;
    auto time_shape = [&](const Shape& sh) -> int {
        if (int r = pmgb_batch_configure(b, sh.n_ctas, sh.order, sh.mflop)) return r;
        if (int r = batch_enqueue(b, seed, temperature)) return r;  // warm-up
        cudaEventRecord(e0, ctx->stream);
        for (int i = 0; i < repeats; ++i)
            if (int r = batch_enqueue(b, seed + 1 + i, temperature)) return r;
        cudaEventRecord(e1, ctx->stream);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "pmgb_batch_tune");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms / repeats < best) {
            best = ms / repeats;
            best_s = sh;
        }
        return PMGB_OK;
    };
    // coordinate search: insertion-tile work per unit, then resident CTAs per SM, then unit order
    for (double mflop : {0.0, 32.0, 128.0, 512.0})
        if (!rc) rc = time_shape(Shape{b->max_ctas, 0, mflop});
    for (int twice : {2, 3})
        if (!rc) rc = time_shape(Shape{std::max(1, twice * b->sm_count / 2), 0, best_s.mflop});
    if (!rc) rc = time_shape(Shape{best_s.n_ctas, 1, best_s.mflop});
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if ((rc = check_status(ctx))) return rc;
    if ((rc = pmgb_batch_configure(b, best_s.n_ctas, best_s.order, best_s.mflop))) return rc;
    if (best_ms_out) *best_ms_out = best;
    return PMGB_OK;
}

extern "C" int pmgb_batch_results(pmgb_batch* b, double* block_out, double* dtheta) {
    if (!b) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = b->ctx;
    if (!block_out || (b->grad && !dtheta))
        return fail(ctx, PMGB_ERR_INVALID_ARGUMENT, "pmgb_batch_results: block_out (and dtheta with the adjoint)");
    if (!b->launched) return fail(ctx, PMGB_ERR_NOT_READY, "pmgb_batch_results: no run since the batch was configured");
    PMGB_CK(ctx, enter_device(ctx->device));
    const size_t nb = b->host_sys.size() * 4 * static_cast<size_t>(b->n_blocks);
    PMGB_CK(ctx, cudaMemcpyAsync(block_out, b->d_block_out, sizeof(double) * nb, cudaMemcpyDeviceToHost, ctx->stream));
    std::vector<double> cols(b->grad ? b->n_out_cols : 0);
    if (b->grad)
        PMGB_CK(ctx, cudaMemcpyAsync(cols.data(), b->d_out_cols, sizeof(double) * cols.size(), cudaMemcpyDeviceToHost,
                                     ctx->stream));
    if (int rc = check_status(ctx)) return rc;
    if (!b->grad) return PMGB_OK;
    double* d = dtheta;
    for (size_t i = 0; i < b->systems.size(); ++i) {
        const pmgb_system* s = b->systems[i];
        const double* c = cols.data() + b->host_sys[i].out_base;
        d[0] = c[0];
        d[1] = c[1];
        d[2] = c[2];
        assemble_species(s, template_sites(s->n_sites), c + 3, d);
        d += 3 + 2 * s->n_species * s->n_species;
    }
    return PMGB_OK;
}

extern "C" int pmgb_batch_refined_counts(pmgb_batch* b, int64_t* per_system) {
    if (!b || !per_system) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = b->ctx;
    for (size_t i = 0; i < b->systems.size(); ++i) per_system[i] = 0;
    if (!(b->refine_tail > 0.0) || !b->launched) return PMGB_OK;
    PMGB_CK(ctx, enter_device(ctx->device));
    std::vector<int> off(static_cast<size_t>(b->n_chunks) + 1);
    PMGB_CK(ctx, cudaMemcpyAsync(off.data(), b->d_offsets, sizeof(int) * off.size(), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    for (size_t i = 0; i < b->host_sys.size(); ++i) {
        const BatchSystem& bs = b->host_sys[i];
        const int64_t c1 = bs.chunk_first + static_cast<int64_t>(bs.ctas_per_block) * b->n_blocks;
        per_system[i] = off[c1] - off[bs.chunk_first];
    }
    return PMGB_OK;
}

extern "C" int pmgb_batch_energies(pmgb_batch* b, double* u_out) {
    if (!b || !u_out) return PMGB_ERR_INVALID_ARGUMENT;
    pmgb_ctx* ctx = b->ctx;
    if (!b->launched || !(b->refine_tail > 0.0 || b->cull) || !b->d_u)
        return fail(ctx, PMGB_ERR_NOT_READY, "pmgb_batch_energies: needs a run with culling or refinement on");
    PMGB_CK(ctx, enter_device(ctx->device));
    PMGB_CK(ctx, cudaMemcpyAsync(u_out, b->d_u, sizeof(double) * 2 * static_cast<size_t>(b->n_insertions),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    PMGB_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return PMGB_OK;
}

extern "C" int pmgb_batch_info(const pmgb_batch* b, int64_t* out8) {
    if (!b || !out8) return PMGB_ERR_INVALID_ARGUMENT;
    out8[0] = static_cast<int64_t>(b->units.size());
    out8[1] = b->n_ctas;
    out8[2] = b->order;
    out8[3] = b->dtheta_len;
    out8[4] = b->device_bytes;
    out8[5] = b->n_insertions;
    out8[6] = b->n_chunks;
    out8[7] = static_cast<int64_t>(std::llround(b->unit_mflop));
    return PMGB_OK;
}

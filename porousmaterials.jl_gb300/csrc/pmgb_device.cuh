// pmgb_device.cuh -- device code shared by the single-system and the batched kernels:
// PTX helpers (mbarrier, 1-D TMA bulk copies), Philox poses, FP32 pair terms, the Ewald
// reciprocal-space recurrence and run_unit, the body that evaluates one CTA-sized unit of
// items against one framework.
//
// One thread owns one insertion (or one grid point / explicit configuration) and
// keeps its guest sites in registers.  Fractional coordinates are 32-bit fixed point
// (x * 2^32 mod 2^32): the wrapping integer difference of two positions is exactly the
// minimum-image fractional displacement (|d| <= 1/2), converted once to FP32 with a
// single rounding.  The CTA streams the replicated framework (species-sorted int4
// records: x, y, z fixed point, q as float bits) through a ring of shared-memory stages filled by
// 1-D TMA bulk copies (cp.async.bulk + mbarrier complete_tx); every thread of the
// CTA reads each record with a broadcast shared load and evaluates it against all
// of its guest sites.  Pair math is FP32; per-insertion sums are compensated
// (TwoSum every 64 records); the Boltzmann accumulation across insertions is FP64
// log-sum-exp.  Ewald reciprocal space uses the framework structure factor
// S(k) = sum_c q_c e^{ik.r_c} (built once per system in FP64) against a per-site
// e^{-ik.x} recurrence along kc.
//
// Reference semantics restated here (PorousMaterials.jl v0.4.2):
//   src/vdw_energetics.jl:19-47   LJ 12-6, strict r^2 < rc^2, r^2 < 0.1 -> +Inf
//   src/electrostatics.jl:347-388 Ewald real space q erfc(alpha r)/(4 pi eps0 r), r < rc,
//                                 reciprocal space sum_k wt_k sum_c q_c cos(k.(r_c - x))
//   src/henry.jl:212-244          Boltzmann factor sums per statistics block, +Inf
//                                 insertions excluded from the weighted-energy sums
//   src/molecule.jl:233-281       uniform random rotation (Arvo) about the centre of mass
//   src/grid.jl:313-359           energy-grid points xf = (i/(n-1), ...) ./ repfactors
#pragma once
#include "pmgb_internal.h"

#include <cmath>
#include <cstdint>

namespace {

constexpr int kChunk = PMGB_CHUNK;      // records per compensated fold
constexpr int kSub = PMGB_SUBCHUNK;     // records per bounding box (a quarter of a chunk)
static_assert(kChunk % kSub == 0 && kSub % 4 == 0 && kChunk / kSub <= 32, "sub-chunks tile a chunk");
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s bound on any mbarrier wait

// ----------------------------------------------------------------------------
// PTX helpers: mbarrier + 1-D bulk (TMA) copies global -> shared
// ----------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Spin on an mbarrier phase for at most limit_ns (and a hard iteration cap).
__device__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                  unsigned long long limit_ns = kWaitLimitNs) {
    unsigned long long t0 = global_ns();
    for (uint32_t it = 0; it < (1u << 28); ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63u) == 63u && global_ns() - t0 > limit_ns) return false;
    }
    return false;
}

// ----------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11)
// ----------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}
__device__ __forceinline__ float u24(uint32_t x) { return static_cast<float>(x >> 8) * 5.9604644775390625e-08f; }

// Index of cell (x, y, z) (2^bits per axis) along a Hilbert curve: the key of the spatial orders
// of Widom runs.  Consecutive cells along the curve share a face, so a run of consecutive
// insertions (a warp's 32, a CTA's 256) stays compact everywhere; along a Z-order curve it can
// straddle a jump across the cell.  J. Skilling, "Programming the Hilbert curve", AIP Conf. Proc.
// 707 (2004): the axes are turned into the transposed index (undo excess work, Gray encode),
// whose bits are then interleaved.
__host__ __device__ __forceinline__ int hilbert_cell(uint32_t cx, uint32_t cy, uint32_t cz, int bits) {
    uint32_t x[3] = {cx, cy, cz};
    for (uint32_t q = 1u << (bits - 1); q > 1u; q >>= 1) {
        const uint32_t p = q - 1u;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (x[i] & q) {
                x[0] ^= p;  // invert the low bits of axis 0
            } else {
                const uint32_t t = (x[0] ^ x[i]) & p;  // exchange the low bits of axes 0 and i
                x[0] ^= t;
                x[i] ^= t;
            }
        }
    }
    x[1] ^= x[0];
    x[2] ^= x[1];
    uint32_t t = 0;
    for (uint32_t q = 1u << (bits - 1); q > 1u; q >>= 1)
        if (x[2] & q) t ^= q - 1u;
    int code = 0;
    for (int b = bits - 1; b >= 0; --b)
        code = code << 3 | static_cast<int>(((x[0] ^ t) >> b & 1u) << 2 | ((x[1] ^ t) >> b & 1u) << 1 | ((x[2] ^ t) >> b & 1u));
    return code;
}

// Pose of Widom insertion `idx`: centre of mass uniform in the supercell's
// fractional cube (henry.jl:214) and a uniform rotation by Arvo's method
// (molecule.jl:233-244): M = -(I - 2 v v^T) Rz(2 pi u1), v from (u2, u3).
// R is column-major (R[i + 3j]).
__device__ __forceinline__ void make_pose(unsigned long long seed, unsigned long long idx, float xf[3],
                                          float R[9]) {
    const uint2 key = make_uint2(static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    const uint4 a = philox4x32_10(make_uint4(static_cast<uint32_t>(idx), static_cast<uint32_t>(idx >> 32), 0u, 0u), key);
    const uint4 b = philox4x32_10(make_uint4(static_cast<uint32_t>(idx), static_cast<uint32_t>(idx >> 32), 1u, 0u), key);
    xf[0] = u24(a.x);
    xf[1] = u24(a.y);
    xf[2] = u24(a.z);
    const float u1 = u24(a.w), u2 = u24(b.x), u3 = u24(b.y);
    float s1, c1, s2, c2;
    sincospif(2.0f * u1, &s1, &c1);
    sincospif(2.0f * u2, &s2, &c2);
    const float sq = sqrtf(u3);
    const float v0 = c2 * sq, v1 = s2 * sq, v2 = sqrtf(1.0f - u3);
    // A = 2 v v^T - I ; M = A * Rz with Rz columns (c1, -s1, 0), (s1, c1, 0), (0, 0, 1)
    // (explicit fused operations throughout, so that every kernel that draws a pose rounds it
    // the same way)
    const float A[3][3] = {{fmaf(2.0f * v0, v0, -1.0f), 2.0f * v0 * v1, 2.0f * v0 * v2},
                           {2.0f * v1 * v0, fmaf(2.0f * v1, v1, -1.0f), 2.0f * v1 * v2},
                           {2.0f * v2 * v0, 2.0f * v2 * v1, fmaf(2.0f * v2, v2, -1.0f)}};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        R[i + 0] = fmaf(A[i][0], c1, -(A[i][1] * s1));
        R[i + 3] = fmaf(A[i][0], s1, A[i][1] * c1);
        R[i + 6] = A[i][2];
    }
}

// ----------------------------------------------------------------------------
// compensated accumulation
// ----------------------------------------------------------------------------
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
    const float s = __fadd_rn(hi, x);
    const float bp = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
    hi = s;
    lo = __fadd_rn(lo, e);
}

// FP32 fractional coordinate -> 32-bit fixed point, wrapping modulo 1
__device__ __forceinline__ uint32_t frac2fix(float x) {
    return static_cast<uint32_t>(__float2ll_rn(x * 4294967296.0f));
}

// FP64 fractional offset (|x| < 1) -> 32-bit fixed point, wrapping modulo 1
__device__ __forceinline__ uint32_t frac2fix64(double x) {
    return static_cast<uint32_t>(__double2ll_rn(x * 4294967296.0));
}

// Guest sites of Widom insertion `item` as fixed-point fractions: the FP32 pose (make_pose;
// its centre of mass is an exact 24-bit fraction) applied to the FP64 site offsets in FP64,
// as the oracle composes them from the same pose.
// com_at (optional): a fixed centre of mass (fixed point) instead of the drawn one; the
// rotation is still the pose's.
template <int NS>
__device__ __forceinline__ void pose_sites(const SysDev& S, unsigned long long seed, unsigned long long item,
                                           uint32_t* ux, uint32_t* uy, uint32_t* uz, float* com = nullptr,
                                           uint32_t* cfix = nullptr, const uint32_t* com_at = nullptr) {
    float xf[3], R[9];
    make_pose(seed, item, xf, R);
    if (com) {
        com[0] = xf[0];
        com[1] = xf[1];
        com[2] = xf[2];
    }
    const uint32_t cx = com_at ? com_at[0] : frac2fix(xf[0]);
    const uint32_t cy = com_at ? com_at[1] : frac2fix(xf[1]);
    const uint32_t cz = com_at ? com_at[2] : frac2fix(xf[2]);
    if (cfix) {
        cfix[0] = cx;
        cfix[1] = cy;
        cfix[2] = cz;
    }
    double r[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) r[i] = static_cast<double>(R[i]);
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        const double bx = S.body64[k][0], by = S.body64[k][1], bz = S.body64[k][2];
        const double ox = fma(r[0], bx, fma(r[3], by, r[6] * bz));
        const double oy = fma(r[1], bx, fma(r[4], by, r[7] * bz));
        const double oz = fma(r[2], bx, fma(r[5], by, r[8] * bz));
        ux[k] = cx + frac2fix64(fma(S.g64[0], ox, fma(S.g64[1], oy, S.g64[2] * oz)));
        uy[k] = cy + frac2fix64(fma(S.g64[3], oy, S.g64[4] * oz));
        uz[k] = cz + frac2fix64(S.g64[5] * oz);
    }
}

// The accessibility gate of src/grid.jl:778-836: the supercell fraction xf scaled by the
// replication factors (mod 1) into the grid's cell, its nearest node 1 + round(x (n - 1))
// (ties to even, as Julia's round), and the node with its 26 neighbours (index 0 -> n,
// n + 1 -> 1); accessible iff any of the 27 is.
__device__ __forceinline__ bool accessible_com(const SysDev& S, const float* xf) {
    int id[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double x = static_cast<double>(xf[d]) * S.acc_rep[d];
        x -= floor(x);
        id[d] = 1 + static_cast<int>(rint(x * (S.acc_n[d] - 1)));
    }
    for (int i = -1; i <= 1; ++i)
        for (int j = -1; j <= 1; ++j)
            for (int k = -1; k <= 1; ++k) {
                int v[3] = {id[0] + i, id[1] + j, id[2] + k};
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    if (v[d] == 0) v[d] = S.acc_n[d];
                    if (v[d] == S.acc_n[d] + 1) v[d] = 1;
                }
                if (S.acc[(v[0] - 1) + static_cast<size_t>(S.acc_n[0]) * ((v[1] - 1) + static_cast<size_t>(S.acc_n[1]) * (v[2] - 1))])
                    return true;
            }
    return false;
}

struct Geo {
    // f_to_c scaled by 2^-32 as an FP32 value h plus its FP32 residual p (h + p equals the
    // FP64 matrix to ~1e-15), so that Cartesian = (h + p) * fixed-point displacement
    float h00, h01, h02, h11, h12, h22;
    float p00, p01, p02, p11, p12, p22;
    float rc2, rc2e, alpha;
};

// erfc(x) for x >= 0: t exp(-x^2) Q(3t - 2) with t = 1/(1 + x/2) and Q the degree-7
// polynomial of csrc/fit_erfc.py (max relative error 3.3e-7 on [0, 3.2]).
__device__ __forceinline__ float erfc_fit(float x) {
    const float t = __fdividef(1.0f, fmaf(0.5f, x, 1.0f));
    const float y = fmaf(t, 3.0f, -2.0f);
    float q = -1.1504688e-05f;
    q = fmaf(q, y, 0.00012701178f);
    q = fmaf(q, y, 1.719709e-05f);
    q = fmaf(q, y, -0.002622572f);
    q = fmaf(q, y, 0.00045600548f);
    q = fmaf(q, y, 0.06661939f);
    q = fmaf(q, y, 0.29403913f);
    q = fmaf(q, y, 0.6413754f);
    float e;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(x * (x * -1.4426950408889634f)));
    return q * t * e;
}

// Cartesian squared distance of a fixed-point fractional displacement
__device__ __forceinline__ float dist2(const int4 r, const uint32_t ux, const uint32_t uy, const uint32_t uz,
                                       const Geo& g) {
    // the wrapping difference is the minimum-image displacement in units of 2^-32
    const float dx = __int2float_rn(static_cast<int>(static_cast<uint32_t>(r.x) - ux));
    const float dy = __int2float_rn(static_cast<int>(static_cast<uint32_t>(r.y) - uy));
    const float dz = __int2float_rn(static_cast<int>(static_cast<uint32_t>(r.z) - uz));
    const float rx = fmaf(g.p00, dx, fmaf(g.p01, dy, g.p02 * dz));
    const float ry = fmaf(g.p11, dy, g.p12 * dz);
    const float rz = g.p22 * dz;
    const float cx = fmaf(g.h00, dx, fmaf(g.h01, dy, fmaf(g.h02, dz, rx)));
    const float cy = fmaf(g.h11, dy, fmaf(g.h12, dz, ry));
    const float cz = fmaf(g.h22, dz, rz);
    return fmaf(cx, cx, fmaf(cy, cy, cz * cz));
}

// One framework record against one guest site.  COLS: also r^-12 and r^-6 within the LJ cutoff
// into *c12, *c6 (the adjoint's columns).
template <bool CHARGED, bool COLS = false>
__device__ __forceinline__ void pair_fwd(const int4 r, const uint32_t ux, const uint32_t uy, const uint32_t uz,
                                         const Geo& g, const float sig2, const float eps4, float& segmin,
                                         float& ljp, float& php, float* c12 = nullptr, float* c6 = nullptr,
                                         float* c24 = nullptr, float* cgap = nullptr) {
    const float r2 = dist2(r, ux, uy, uz, g);
    segmin = fminf(segmin, r2);
    if (cgap) *cgap = fminf(*cgap, fabsf(r2 - g.rc2));  // error bound: distance to the LJ cutoff
    const bool in = r2 < g.rc2;
    float ir2, y = 0.0f;
    if (CHARGED) {
        // rsqrt estimate refined by one Newton step: y <- y + y/2 (1 - r2 y^2)
        y = rsqrtf(r2);
        const float e = fmaf(-r2 * y, y, 1.0f);
        y = fmaf(0.5f * y, e, y);
        ir2 = y * y;
    } else {
        ir2 = __frcp_rn(r2);
    }
    const float s = sig2 * ir2;
    const float s3 = s * s * s;
    const float t = fmaf(s3, s3, -s3);
    ljp = fmaf(eps4, in ? t : 0.0f, ljp);
    if (COLS) {
        const float ir6 = in ? ir2 * ir2 * ir2 : 0.0f;
        const float ir12 = ir6 * ir6;
        *c12 += ir12;
        *c6 += ir6;
        if (c24) *c24 = fmaf(ir12, ir12, *c24);
    }
    if (CHARGED) {
        const float e = erfc_fit(g.alpha * (r2 * y)) * y;
        php = fmaf(__int_as_float(r.w), (r2 < g.rc2e) ? e : 0.0f, php);
    }
}

// ---- packed (f32x2) form: two framework records against one guest site -------------
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float ex2_approx(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

struct Geo2 {
    float2 h00, h01, h02, h11, h12, h22;
    float2 p00, p01, p02, p11, p12, p22;
    float rc2, rc2e;
    float rcmax2;        // the larger cutoff^2: beyond it a pair contributes nothing
    float2 half_alpha;   // alpha / 2
    float2 m_a2_log2e;   // -alpha^2 log2(e)
};

// erfc(alpha r) from r and r^2 (see erfc_fit; t = 1/(1 + alpha r/2), exp(-alpha^2 r^2) = 2^(c r^2))
__device__ __forceinline__ float2 erfc_fit2(float2 r, float2 r2, const Geo2& g) {
    const float2 a = fma2(g.half_alpha, r, f2(1.0f));
    const float2 t = make_float2(rcp_approx(a.x), rcp_approx(a.y));
    const float2 y = fma2(t, f2(3.0f), f2(-2.0f));
    float2 q = f2(-1.1504688e-05f);
    q = fma2(q, y, f2(0.00012701178f));
    q = fma2(q, y, f2(1.719709e-05f));
    q = fma2(q, y, f2(-0.002622572f));
    q = fma2(q, y, f2(0.00045600548f));
    q = fma2(q, y, f2(0.06661939f));
    q = fma2(q, y, f2(0.29403913f));
    q = fma2(q, y, f2(0.6413754f));
    const float2 arg = mul2(g.m_a2_log2e, r2);
    return mul2(mul2(q, t), make_float2(ex2_approx(arg.x), ex2_approx(arg.y)));
}

// erfc(alpha r) and exp(-alpha^2 r^2), for the adjoint
__device__ __forceinline__ float2 erfc_fit2_exp(float2 r, float2 r2, const Geo2& g, float2& ex) {
    const float2 a = fma2(g.half_alpha, r, f2(1.0f));
    const float2 t = make_float2(rcp_approx(a.x), rcp_approx(a.y));
    const float2 y = fma2(t, f2(3.0f), f2(-2.0f));
    float2 q = f2(-1.1504688e-05f);
    q = fma2(q, y, f2(0.00012701178f));
    q = fma2(q, y, f2(1.719709e-05f));
    q = fma2(q, y, f2(-0.002622572f));
    q = fma2(q, y, f2(0.00045600548f));
    q = fma2(q, y, f2(0.06661939f));
    q = fma2(q, y, f2(0.29403913f));
    q = fma2(q, y, f2(0.6413754f));
    const float2 arg = mul2(g.m_a2_log2e, r2);
    ex = make_float2(ex2_approx(arg.x), ex2_approx(arg.y));
    return mul2(mul2(q, t), ex);
}

// Per (record pair, site) adjoint accumulators
struct Grad2 {
    float2 i12, i6;        // sum r^-12, sum r^-6 within the LJ cutoff
    float2 gx, gy, gz;     // sum c (dU/dr^2) with the site's charge folded into the Coulomb part
};

// The forward pair terms plus the adjoint ones.  c = x_framework - x_site (Cartesian, the
// frame of the upper-triangular box); dU/dx_site = -2 sum_j c_j dU_j/d(r^2).
template <bool CHARGED>
__device__ __forceinline__ void pair2_grad(const int4 ra, const int4 rb, const uint32_t ux, const uint32_t uy,
                                           const uint32_t uz, const Geo2& g, const float2 lj12, const float2 lj6,
                                           const float2 qcoul, const float2 c1, const float2 lane_mask,
                                           float& segmin, float2& ljp, float2& php, Grad2& G) {
    const float2 dx = make_float2(__int2float_rn(static_cast<int>(static_cast<uint32_t>(ra.x) - ux)),
                                  __int2float_rn(static_cast<int>(static_cast<uint32_t>(rb.x) - ux)));
    const float2 dy = make_float2(__int2float_rn(static_cast<int>(static_cast<uint32_t>(ra.y) - uy)),
                                  __int2float_rn(static_cast<int>(static_cast<uint32_t>(rb.y) - uy)));
    const float2 dz = make_float2(__int2float_rn(static_cast<int>(static_cast<uint32_t>(ra.z) - uz)),
                                  __int2float_rn(static_cast<int>(static_cast<uint32_t>(rb.z) - uz)));
    const float2 rx = fma2(g.p00, dx, fma2(g.p01, dy, mul2(g.p02, dz)));
    const float2 ry = fma2(g.p11, dy, mul2(g.p12, dz));
    const float2 rz = mul2(g.p22, dz);
    const float2 cx = fma2(g.h00, dx, fma2(g.h01, dy, fma2(g.h02, dz, rx)));
    const float2 cy = fma2(g.h11, dy, fma2(g.h12, dz, ry));
    const float2 cz = fma2(g.h22, dz, rz);
    const float2 r2 = fma2(cx, cx, fma2(cy, cy, mul2(cz, cz)));
    segmin = fminf(segmin, fminf(r2.x, r2.y));
    float2 ir2, y = f2(0.0f);
    if (CHARGED) {
        y = make_float2(rsqrt_approx(r2.x), rsqrt_approx(r2.y));
        const float2 hy = mul2(f2(-0.5f), mul2(r2, y));
        y = fma2(y, fma2(hy, y, f2(0.5f)), y);
        ir2 = mul2(y, y);
    } else {
        const float2 r0 = make_float2(rcp_approx(r2.x), rcp_approx(r2.y));
        const float2 e = fma2(mul2(f2(-1.0f), r2), r0, f2(1.0f));
        ir2 = fma2(r0, e, r0);
    }
    const float2 ir6 = mul2(mul2(ir2, ir2), ir2);
    const float2 ir6c = mul2(lane_mask, make_float2(r2.x < g.rc2 ? ir6.x : 0.0f, r2.y < g.rc2 ? ir6.y : 0.0f));
    const float2 ir12c = mul2(ir6c, ir6c);
    ljp = fma2(ir6c, fma2(lj12, ir6c, lj6), ljp);
    G.i12 = __fadd2_rn(G.i12, ir12c);
    G.i6 = __fadd2_rn(G.i6, ir6c);
    // dU_LJ/d(r^2) = -r^-2 r^-6 (6 lj12 r^-6 + 3 lj6)
    float2 du = mul2(mul2(f2(-1.0f), ir2), mul2(ir6c, fma2(mul2(f2(6.0f), lj12), ir6c, mul2(f2(3.0f), lj6))));
    if (CHARGED) {
        const float2 rr = mul2(r2, y);
        float2 ex;
        const float2 erfcv = erfc_fit2_exp(rr, r2, g, ex);
        const float2 e = mul2(erfcv, y);
        const float2 qj = make_float2(__int_as_float(ra.w), __int_as_float(rb.w));
        const float2 in_e = mul2(lane_mask, make_float2(r2.x < g.rc2e ? 1.0f : 0.0f, r2.y < g.rc2e ? 1.0f : 0.0f));
        php = fma2(mul2(qj, in_e), e, php);
        // d(q_j erfc(a r)/r)/d(r^2) = -q_j r^-2 / 2 [c1 exp(-a^2 r^2) + erfc(a r)/r], c1 = 2a/sqrt(pi)
        const float2 dc = mul2(mul2(mul2(f2(-0.5f), mul2(qj, in_e)), ir2), fma2(c1, ex, e));
        du = fma2(qcoul, dc, du);
    }
    G.gx = fma2(cx, du, G.gx);
    G.gy = fma2(cy, du, G.gy);
    G.gz = fma2(cz, du, G.gz);
}

// Squared minimum-image distances of two records from one guest site.
// RESID = false: the FP32 box matrix alone (its rounding, ~6e-8 relative, biases every distance
// of a system the same way; used only where an FP64 refinement follows)
template <bool RESID = true>
__device__ __forceinline__ float2 pair2_r2(const int4 ra, const int4 rb, const uint32_t ux, const uint32_t uy,
                                           const uint32_t uz, const Geo2& g) {
    const float2 dx = make_float2(__int2float_rn(static_cast<int>(static_cast<uint32_t>(ra.x) - ux)),
                                  __int2float_rn(static_cast<int>(static_cast<uint32_t>(rb.x) - ux)));
    const float2 dy = make_float2(__int2float_rn(static_cast<int>(static_cast<uint32_t>(ra.y) - uy)),
                                  __int2float_rn(static_cast<int>(static_cast<uint32_t>(rb.y) - uy)));
    const float2 dz = make_float2(__int2float_rn(static_cast<int>(static_cast<uint32_t>(ra.z) - uz)),
                                  __int2float_rn(static_cast<int>(static_cast<uint32_t>(rb.z) - uz)));
    if (!RESID) {
        const float2 cx = fma2(g.h00, dx, fma2(g.h01, dy, mul2(g.h02, dz)));
        const float2 cy = fma2(g.h11, dy, mul2(g.h12, dz));
        const float2 cz = mul2(g.h22, dz);
        return fma2(cx, cx, fma2(cy, cy, mul2(cz, cz)));
    }
    const float2 rx = fma2(g.p00, dx, fma2(g.p01, dy, mul2(g.p02, dz)));
    const float2 ry = fma2(g.p11, dy, mul2(g.p12, dz));
    const float2 rz = mul2(g.p22, dz);
    const float2 cx = fma2(g.h00, dx, fma2(g.h01, dy, fma2(g.h02, dz, rx)));
    const float2 cy = fma2(g.h11, dy, fma2(g.h12, dz, ry));
    const float2 cz = fma2(g.h22, dz, rz);
    return fma2(cx, cx, fma2(cy, cy, mul2(cz, cz)));
}

// Cartesian minimum-image displacements of two records from the guest's pose centre (fixed
// point cx, cy, cz), converted once per record for all guest sites (the centre-image path),
// with the box-matrix residual.
__device__ __forceinline__ void com_disp2(const int4 ra, const int4 rb, const uint32_t cx, const uint32_t cy,
                                          const uint32_t cz, const Geo2& g, float2& X, float2& Y, float2& Z) {
    const float2 dx = make_float2(__int2float_rn(static_cast<int>(static_cast<uint32_t>(ra.x) - cx)),
                                  __int2float_rn(static_cast<int>(static_cast<uint32_t>(rb.x) - cx)));
    const float2 dy = make_float2(__int2float_rn(static_cast<int>(static_cast<uint32_t>(ra.y) - cy)),
                                  __int2float_rn(static_cast<int>(static_cast<uint32_t>(rb.y) - cy)));
    const float2 dz = make_float2(__int2float_rn(static_cast<int>(static_cast<uint32_t>(ra.z) - cz)),
                                  __int2float_rn(static_cast<int>(static_cast<uint32_t>(rb.z) - cz)));
    const float2 rx = fma2(g.p00, dx, fma2(g.p01, dy, mul2(g.p02, dz)));
    const float2 ry = fma2(g.p11, dy, mul2(g.p12, dz));
    const float2 rz = mul2(g.p22, dz);
    X = fma2(g.h00, dx, fma2(g.h01, dy, fma2(g.h02, dz, rx)));
    Y = fma2(g.h11, dy, fma2(g.h12, dz, ry));
    Z = fma2(g.h22, dz, rz);
}

// Squared distances of a guest site from two records, given the records' displacements from
// the pose centre and the site's negated Cartesian offset (nx, ny, nz).
__device__ __forceinline__ float2 site_r2(const float2 X, const float2 Y, const float2 Z, const float nx,
                                          const float ny, const float nz) {
    const float2 ex = __fadd2_rn(X, f2(nx)), ey = __fadd2_rn(Y, f2(ny)), ez = __fadd2_rn(Z, f2(nz));
    return fma2(ex, ex, fma2(ey, ey, mul2(ez, ez)));
}

// LJ and real-space terms of two records at squared distances r2 (charges qa, qb); COLS: also
// r^-12 and r^-6 within the LJ cutoff into *c12, *c6.
template <bool CHARGED, bool COLS = false>
__device__ __forceinline__ void pair2_energy(const float2 r2, const float qa, const float qb, const Geo2& g,
                                             const float2 lj12, const float2 lj6, float2& ljp, float2& php,
                                             float2* c12 = nullptr, float2* c6 = nullptr, float2* c24 = nullptr) {
    float2 ir2, y = f2(0.0f);
    if (CHARGED) {
        y = make_float2(rsqrt_approx(r2.x), rsqrt_approx(r2.y));
        const float2 hy = mul2(f2(-0.5f), mul2(r2, y));
        y = fma2(y, fma2(hy, y, f2(0.5f)), y);
        ir2 = mul2(y, y);
    } else {
        const float2 r0 = make_float2(rcp_approx(r2.x), rcp_approx(r2.y));
        const float2 e = fma2(mul2(f2(-1.0f), r2), r0, f2(1.0f));
        ir2 = fma2(r0, e, r0);
    }
    const float2 ir6 = mul2(mul2(ir2, ir2), ir2);
    const float2 ir6c = make_float2(r2.x < g.rc2 ? ir6.x : 0.0f, r2.y < g.rc2 ? ir6.y : 0.0f);
    ljp = fma2(ir6c, fma2(lj12, ir6c, lj6), ljp);
    if (COLS) {
        const float2 ir12c = mul2(ir6c, ir6c);
        *c12 = __fadd2_rn(*c12, ir12c);
        *c6 = __fadd2_rn(*c6, ir6c);
        if (c24) *c24 = fma2(ir12c, ir12c, *c24);
    }
    if (CHARGED) {
        const float2 rr = mul2(r2, y);
        const float2 e = mul2(erfc_fit2(rr, r2, g), y);
        php = fma2(make_float2(qa, qb), make_float2(r2.x < g.rc2e ? e.x : 0.0f, r2.y < g.rc2e ? e.y : 0.0f), php);
    }
}

template <bool CHARGED, bool RESID = true, bool COLS = false>
__device__ __forceinline__ void pair2_fwd(const int4 ra, const int4 rb, const uint32_t ux, const uint32_t uy,
                                          const uint32_t uz, const Geo2& g, const float2 lj12, const float2 lj6,
                                          float& segmin, float2& ljp, float2& php, float2* c12 = nullptr,
                                          float2* c6 = nullptr) {
    const float2 r2 = pair2_r2<RESID>(ra, rb, ux, uy, uz, g);  // the same distances as the culled loop
    segmin = fminf(segmin, fminf(r2.x, r2.y));
    float2 ir2, y = f2(0.0f);
    if (CHARGED) {
        // rsqrt estimate refined by one Newton step: y <- y + y (1/2 - (r2/2) y^2)
        y = make_float2(rsqrt_approx(r2.x), rsqrt_approx(r2.y));
        const float2 hy = mul2(f2(-0.5f), mul2(r2, y));
        y = fma2(y, fma2(hy, y, f2(0.5f)), y);
        ir2 = mul2(y, y);
    } else {
        const float2 r0 = make_float2(rcp_approx(r2.x), rcp_approx(r2.y));
        const float2 e = fma2(mul2(f2(-1.0f), r2), r0, f2(1.0f));
        ir2 = fma2(r0, e, r0);
    }
    // 4 eps [(s2/r2)^6 - (s2/r2)^3] = ir6 (lj12 ir6 - lj6), ir6 zeroed beyond the cutoff
    const float2 ir6 = mul2(mul2(ir2, ir2), ir2);
    const float2 ir6c = make_float2(r2.x < g.rc2 ? ir6.x : 0.0f, r2.y < g.rc2 ? ir6.y : 0.0f);
    ljp = fma2(ir6c, fma2(lj12, ir6c, lj6), ljp);
    if (COLS) {
        *c12 = __fadd2_rn(*c12, mul2(ir6c, ir6c));
        *c6 = __fadd2_rn(*c6, ir6c);
    }
    if (CHARGED) {
        const float2 rr = mul2(r2, y);
        const float2 e = mul2(erfc_fit2(rr, r2, g), y);
        php = fma2(make_float2(__int_as_float(ra.w), __int_as_float(rb.w)),
                   make_float2(r2.x < g.rc2e ? e.x : 0.0f, r2.y < g.rc2e ? e.y : 0.0f), php);
    }
}

// Reciprocal-space energy of the whole guest, sum_k Re[wt_k S(k) G(k)] with
// G(k) = sum_g q_g e^{-ik.x_g} = e^{-ik.x_0} (q_tot + sum_g q_g (e^{-ik.(x_g - x_0)} - 1)).
// Combining the guest's charges per k before multiplying by the (large) wt_k S(k) keeps
// the sum free of the cancellation between per-site potentials of a neutral molecule;
// D_g = e^{-ik.d_g} - 1 is carried by the recurrence D <- D w + (w - 1), whose error is
// relative to |D|.  Phases are exact 32-bit fixed-point turns.  Rows of constant (ka, kb)
// start at the kc nearest 0 and step outward in kc by `dir`.
template <int NS, bool GRAD = false>
__device__ __forceinline__ void kspace_fwd(const SysDev& S, const uint32_t Ua_in[NS], const uint32_t Ub_in[NS],
                                           const uint32_t Uc_in[NS], float& plr_hi, float& plr_lo,
                                           float (*gu)[3] = nullptr, int row0 = 0, int row_step = 1) {
    // GRAD: gu[g][d] receives dU_lr/du_g (fractional coordinates of site g)
    constexpr float kTurn = 4.656612873077393e-10f;  // 2^-31: int32 fixed point -> half turns
    plr_hi = 0.0f;
    plr_lo = 0.0f;
    // rows hold k / ks: evaluate them at ks u (exact in fixed point, modulo one cell)
    uint32_t Ua[NS], Ub[NS], Uc[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        Ua[k] = static_cast<uint32_t>(S.ks[0]) * Ua_in[k];
        Ub[k] = static_cast<uint32_t>(S.ks[1]) * Ub_in[k];
        Uc[k] = static_cast<uint32_t>(S.ks[2]) * Uc_in[k];
    }
    // offsets of sites 1.. from site 0 (exact small integers) and their charges
    int da[NS], db[NS], dc[NS];
    float qg[NS];
    float qtot = 0.0f;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        da[k] = static_cast<int>(Ua[k] - Ua[0]);
        db[k] = static_cast<int>(Ub[k] - Ub[0]);
        dc[k] = static_cast<int>(Uc[k] - Uc[0]);
        qg[k] = (k < S.n_sites) ? S.q[k] : 0.0f;
        qtot += qg[k];
    }
    // step factors along +kc: w0 = e^{-2 pi i uc0} for site 0; for site g: wd = e^{-2 pi i dc_g},
    // dw = wd - 1 = (-2 sin^2(pi dc), -sin(2 pi dc)) evaluated without cancellation
    float w0r, w0i;
    {
        float sn, cs;
        sincospif(static_cast<float>(static_cast<int32_t>(Uc[0])) * kTurn, &sn, &cs);
        w0r = cs;
        w0i = -sn;
    }
    if (NS == 3 && !GRAD && S.k_mirror) {
        // sites 1 and 2 mirror each other through site 0 with equal charges: d_2 = -d_1 exactly,
        // so D_2 = conj(D_1) and H = q_tot + 2 q_1 Re D_1 is real; part += Re[T] H.  Half the
        // work per k-vector of the general loop below (which gives the same sum up to rounding)
        const float q2 = 2.0f * qg[1];
        float sn, cs;
        sincospif(static_cast<float>(dc[1]) * (0.5f * kTurn), &sn, &cs);  // half angle
        const float dwr = -2.0f * sn * sn, dwi = -2.0f * sn * cs;
        const float wdr = __fadd_rn(1.0f, dwr);
        for (int row = row0; row < S.n_krow; row += row_step) {
            const KRow R = S.krow[row];
            const float sgn = static_cast<float>(R.dir);
            float er, ei;
            {
                const uint32_t P = static_cast<uint32_t>(R.ka) * Ua[0] + static_cast<uint32_t>(R.kb) * Ub[0] +
                                   static_cast<uint32_t>(R.kc0) * Uc[0];
                float s0, c0;
                sincospif(static_cast<float>(static_cast<int32_t>(P)) * kTurn, &s0, &c0);
                er = c0;
                ei = -s0;
            }
            float Dr, Di;
            {
                const uint32_t p = static_cast<uint32_t>(R.ka) * static_cast<uint32_t>(da[1]) +
                                   static_cast<uint32_t>(R.kb) * static_cast<uint32_t>(db[1]) +
                                   static_cast<uint32_t>(R.kc0) * static_cast<uint32_t>(dc[1]);
                float s1, c1;
                sincospif(static_cast<float>(static_cast<int32_t>(p)) * (0.5f * kTurn), &s1, &c1);
                Dr = -2.0f * s1 * s1;
                Di = -2.0f * s1 * c1;
            }
            const float sw0i = sgn * w0i, swdi = sgn * dwi;
            float part = 0.0f;
            const float2* sw = S.skw + R.off;
            for (int m = 0; m < R.n; ++m) {
                const float2 w = __ldg(sw + m);
                const float hr = fmaf(q2, Dr, qtot);
                const float tr = fmaf(w.x, er, -w.y * ei);
                part = fmaf(tr, hr, part);
                const float nr = fmaf(er, w0r, -ei * sw0i);
                ei = fmaf(er, sw0i, ei * w0r);
                er = nr;
                const float dr2 = fmaf(Dr, wdr, fmaf(-Di, swdi, dwr));
                Di = fmaf(Dr, swdi, fmaf(Di, wdr, swdi));
                Dr = dr2;
            }
            two_sum_acc(plr_hi, plr_lo, part);
        }
        return;
    }
    float wdr[NS], wdi[NS], dwr[NS], dwi[NS];
#pragma unroll
    for (int k = 1; k < NS; ++k) {
        float sn, cs;
        sincospif(static_cast<float>(dc[k]) * (0.5f * kTurn), &sn, &cs);  // half angle
        dwr[k] = -2.0f * sn * sn;
        dwi[k] = -2.0f * sn * cs;
        wdr[k] = __fadd_rn(1.0f, dwr[k]);  // not fused: the same rounding in every kernel
        wdi[k] = dwi[k];
    }
    for (int row = row0; row < S.n_krow; row += row_step) {
        const KRow R = S.krow[row];
        const float sgn = static_cast<float>(R.dir);  // +1 or -1: direction along kc
        // site-0 phasor at the row start
        float er, ei;
        {
            const uint32_t P = static_cast<uint32_t>(R.ka) * Ua[0] + static_cast<uint32_t>(R.kb) * Ub[0] +
                               static_cast<uint32_t>(R.kc0) * Uc[0];
            float sn, cs;
            sincospif(static_cast<float>(static_cast<int32_t>(P)) * kTurn, &sn, &cs);
            er = cs;
            ei = -sn;
        }
        const float sw0i = sgn * w0i;  // conj for the downward direction
        float Dr[NS], Di[NS], swdi[NS], sdwi[NS];
#pragma unroll
        for (int k = 1; k < NS; ++k) {
            // k.d_g in fixed point, modulo one turn (a wrap flips the signs of both sn and cs,
            // which leaves D unchanged)
            const uint32_t p = static_cast<uint32_t>(R.ka) * static_cast<uint32_t>(da[k]) +
                               static_cast<uint32_t>(R.kb) * static_cast<uint32_t>(db[k]) +
                               static_cast<uint32_t>(R.kc0) * static_cast<uint32_t>(dc[k]);
            float sn, cs;
            sincospif(static_cast<float>(static_cast<int32_t>(p)) * (0.5f * kTurn), &sn, &cs);  // half angle
            Dr[k] = -2.0f * sn * sn;
            Di[k] = -2.0f * sn * cs;
            swdi[k] = sgn * wdi[k];
            sdwi[k] = sgn * dwi[k];
        }
        float part = 0.0f;
        float vs[NS], vk[NS];  // GRAD: sum_m Im[T E_g] and sum_m kc Im[T E_g] along the row
#pragma unroll
        for (int k = 0; k < NS; ++k) vs[k] = vk[k] = 0.0f;
        float kcf = static_cast<float>(R.kc0);
        const float2* sw = S.skw + R.off;
        for (int m = 0; m < R.n; ++m) {
            const float2 w = __ldg(sw + m);
            // H = q_tot + sum_g q_g D_g
            float hr = qtot, hi = 0.0f;
#pragma unroll
            for (int k = 1; k < NS; ++k) {
                hr = fmaf(qg[k], Dr[k], hr);
                hi = fmaf(qg[k], Di[k], hi);
            }
            // T = wt S e^{-ik.x0};  part += Re[T H]
            const float tr = fmaf(w.x, er, -w.y * ei);
            const float ti = fmaf(w.x, ei, w.y * er);
            part = fmaf(tr, hr, fmaf(-ti, hi, part));
            if (GRAD) {
                // Im[T (1 + D_g)] for every site (D_0 = 0)
#pragma unroll
                for (int k = 0; k < NS; ++k) {
                    const float v = (k == 0) ? ti : fmaf(tr, Di[k], fmaf(ti, Dr[k], ti));
                    vs[k] += v;
                    vk[k] = fmaf(kcf, v, vk[k]);
                }
                kcf += sgn;
            }
            // advance one step in kc
            const float nr = fmaf(er, w0r, -ei * sw0i);
            ei = fmaf(er, sw0i, ei * w0r);
            er = nr;
#pragma unroll
            for (int k = 1; k < NS; ++k) {
                const float dr2 = fmaf(Dr[k], wdr[k], fmaf(-Di[k], swdi[k], dwr[k]));
                Di[k] = fmaf(Dr[k], swdi[k], fmaf(Di[k], wdr[k], sdwi[k]));
                Dr[k] = dr2;
            }
        }
        two_sum_acc(plr_hi, plr_lo, part);
        if (GRAD) {
            // dU/du_g = 2 pi q_g sum_k k Im[T E_g]
#pragma unroll
            for (int k = 0; k < NS; ++k) {
                const float f = 6.283185307179586f * qg[k];
                gu[k][0] = fmaf(f * static_cast<float>(R.ka * S.ks[0]), vs[k], gu[k][0]);
                gu[k][1] = fmaf(f * static_cast<float>(R.kb * S.ks[1]), vs[k], gu[k][1]);
                gu[k][2] = fmaf(f * static_cast<float>(S.ks[2]), vk[k], gu[k][2]);
            }
        }
    }
}

// ----------------------------------------------------------------------------
// One CTA-sized unit of work: PMGB_THREADS items (insertions, configurations or grid
// points) of one system against its whole framework.  Used once per CTA by the
// single-system kernels and repeatedly by the persistent batch kernel.
// ----------------------------------------------------------------------------
// Log-sum-exp Boltzmann partial of one CTA: every thread passes its x = -U/T (-inf: no
// insertion or U = +Inf), U_vdw, U_es and overlap count; thread 0 of warp 0 writes
// (max x, sum e^{x - max}, sum U_vdw e^{..}, sum U_es e^{..}, n_inf).  A fixed shuffle tree,
// so the partial depends only on which insertions the CTA holds.
__device__ __forceinline__ void lse_cta(double x, double ev, double ee, long long ninf, LsePartial* red,
                                        LsePartial* partial, double* m_out) {
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    const unsigned full = 0xffffffffu;
    double m = x;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(full, m, o));
    double w = (m == -inf || x == -inf) ? 0.0 : exp(x - m);
    double s = w, tv = w * ev, te = w * ee;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(full, s, o);
        tv += __shfl_xor_sync(full, tv, o);
        te += __shfl_xor_sync(full, te, o);
        ninf += __shfl_xor_sync(full, ninf, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = LsePartial{m, s, tv, te, ninf, 0};
    __syncthreads();
    if (warp == 0) {
        constexpr int NW = PMGB_THREADS / 32;
        LsePartial p = (lane < NW) ? red[lane] : LsePartial{-inf, 0.0, 0.0, 0.0, 0, 0};
        double M = p.m;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) M = fmax(M, __shfl_xor_sync(full, M, o));
        const double f = (M == -inf || p.m == -inf) ? 0.0 : exp(p.m - M);
        double s2 = p.s * f, tv2 = p.tv * f, te2 = p.te * f;
        long long n2 = p.n_inf;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s2 += __shfl_xor_sync(full, s2, o);
            tv2 += __shfl_xor_sync(full, tv2, o);
            te2 += __shfl_xor_sync(full, te2, o);
            n2 += __shfl_xor_sync(full, n2, o);
        }
        if (lane == 0) {
            *partial = LsePartial{M, s2, tv2, te2, n2, 0};
            if (m_out) *m_out = M;
        }
    }
}

struct UnitIO {
    int pose_mode, out_mode;
    long long item;              // this thread's item index within its system
    bool valid;
    // POSE_PHILOX on a grid (rotational energy grids): the centre of mass is the grid point of
    // the item's block, com_at (fixed point); the rotation comes from Philox counter item + item_base
    bool at_point;
    uint32_t com_at[3];
    long long item_base;
    unsigned long long seed;     // POSE_PHILOX
    double inv_temperature;
    const uint32_t* site_fix;    // POSE_SITES
    const uint32_t *grid_x, *grid_y, *grid_z;  // POSE_GRID
    int n1, n2;
    double* u_out;               // per item (U_vdw, U_es) (or U for grids in GRAD)
    double* e_out;               // OUT_ENERGY
    float* grid_out;             // OUT_GRID
    float unit_factor;
    float* dsum;                 // GRAD columns: dsum[c * dsum_stride + col_item]
    long long dsum_stride, col_item;
    float* grad_u;               // GRAD, optional
    float* bound_out;            // OUT_GRID with BOUND: per-item FP32 error estimate (+Inf: must be refined)
    float bound_rho, bound_stat; // BOUND: worst-case per-term factor, statistical factor (see run_unit)
    unsigned long long* stats;   // STATS: [3] distances evaluated, LJ and real-space terms inside their cutoffs
    LsePartial* partial;         // OUT_WIDOM: this unit's partial
    double* x_out;               // OUT_WIDOM, optional: this thread's -U/T (-inf if none)
    double* m_out;               // OUT_WIDOM, optional (shared): the unit's max of -U/T
    bool resident;               // the ring already holds this framework (n_tiles <= PMGB_NSTAGE)
    bool cull;                   // the warp's items are spatially ordered: skip out-of-cutoff terms
};

// Fixed-point gap between a site and a chunk box along one axis: |wrap(c - u)| - e, at least 0.
// The circular distance obeys the triangle inequality, so every record of the chunk lies at
// least this far (in fractions of the axis) from the site along that axis, in its nearest image.
__device__ __forceinline__ float box_gap(uint32_t c, uint32_t u, uint32_t e) {
    const int d = static_cast<int>(c - u);
    const uint32_t a = d < 0 ? 0u - static_cast<uint32_t>(d) : static_cast<uint32_t>(d);
    return a > e ? static_cast<float>(a - e) : 0.0f;
}

// Can any lane of the warp have a site within the cutoff of a record of sub-chunk box B?  A record
// at fractional gaps g_d (per axis, nearest image) lies at least g_d W_d from the site along the
// unit normal n_d of face d (W_d: perpendicular width), so its distance r satisfies
// r^2 >= max_d (g_d W_d)^2 and r^2 >= sum_d (g_d W_d)^2 / lambda_max(n_i . n_j).  The chunk is
// skipped when that bound exceeds the cutoff by 1e-4 relative (far above FP32 rounding): every
// pair term of it would be an exact zero, so the sums do not change.
template <int NS>
__device__ __forceinline__ bool chunk_near(const SysDev& S, const ChunkBox* box, const uint32_t* ux,
                                           const uint32_t* uy, const uint32_t* uz, bool active, float rcmax2) {
    const uint4 c = __ldg(reinterpret_cast<const uint4*>(box));
    const uint4 e = __ldg(reinterpret_cast<const uint4*>(box) + 1);
    bool near = false;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        if (k < S.n_sites) {
            const float gx = box_gap(c.x, ux[k], e.x) * S.cw[0];
            const float gy = box_gap(c.y, uy[k], e.y) * S.cw[1];
            const float gz = box_gap(c.z, uz[k], e.z) * S.cw[2];
            const float sum = fmaf(gx, gx, fmaf(gy, gy, gz * gz)) * S.cw_inv_lam;
            const float mx = fmaxf(fmaxf(gx * gx, gy * gy), gz * gz);
            near = near || fmaxf(sum, mx) <= rcmax2 * 1.0001f;
        }
    }
    return __any_sync(0xffffffffu, active && near);
}

// The same test for the centre-image path, from the pose centre: a record at distance r from the
// centre lies at least r - com_reach from every guest site, so the sub-chunk can matter only if
// the bound on r is within cutoff + com_reach (S.com_reach2 its square).
__device__ __forceinline__ bool chunk_near_com(const SysDev& S, const ChunkBox* box, const uint32_t* cfix,
                                               bool active) {
    const uint4 c = __ldg(reinterpret_cast<const uint4*>(box));
    const uint4 e = __ldg(reinterpret_cast<const uint4*>(box) + 1);
    const float gx = box_gap(c.x, cfix[0], e.x) * S.cw[0];
    const float gy = box_gap(c.y, cfix[1], e.y) * S.cw[1];
    const float gz = box_gap(c.z, cfix[2], e.z) * S.cw[2];
    const float sum = fmaf(gx, gx, fmaf(gy, gy, gz * gz)) * S.cw_inv_lam;
    const float mx = fmaxf(fmaxf(gx * gx, gy * gy), gz * gz);
    return __any_sync(0xffffffffu, active && fmaxf(sum, mx) <= S.com_reach2 * 1.0001f);
}

// Returns false if a bounded wait gave up (the status word is set); every thread of the CTA
// returns the same value.  fills[s] counts the completed fills of ring slot s so far; the
// caller keeps it across units (the barriers are initialised once per CTA).
// GRAD: the adjoint's per-(segment, site) columns sum r^-12, sum r^-6; FORCES (with GRAD): also
// dU/dx per item.  Without FORCES the adjoint runs the forward loops with the columns added, so
// its energies are the forward kernel's.  COMP: the centre-image path (Widom poses of a guest
// with several sites where S.com_axis >= -1; the caller checks both).
// BOUND (energy grids of uncharged probes): also an estimate of the item's FP32 rounding error,
// written to io.bound_out for the screen that picks the items to re-evaluate in double-float.
// With rep, att the r^-12 and r^-6 magnitudes of each LJ term inside the cutoff,
// B = sum (rep + att) and Q = sum (rep^2 + att^2):
//   E = min(bound_rho B, bound_stat sqrt(Q)) + 2e-8 B,
// the first a worst-case bound of the per-term rounding, the second a multiple of the rms of
// independent per-term roundings, the last the 2^-32 quantisation of the item's position; +Inf
// when some pair sits within FP32 rounding of the cutoff or of the overlap distance (the two
// sides of either give different energies).  Runs the spatially culled loop.
// STATS (a diagnostic of the work done, for the counted-work roofline): the loops also count, per
// valid item, the (record, site) distances evaluated -- records of skipped sub-chunks are not --
// and the pairs inside the LJ and real-space cutoffs, added into io.stats[0..2].
template <int NS, bool CHARGED, bool GRAD, bool RESID = true, bool FORCES = GRAD, bool COMP = false,
          bool BOUND = false, bool STATS = false>
__device__ __forceinline__ bool run_unit(const SysDev& S, const UnitIO& io, int4* stage, uint64_t* bars,
                                         LsePartial* red, uint32_t (&fills)[PMGB_NSTAGE], unsigned int* status) {
    static_assert(RESID || !GRAD, "the adjoint keeps the box-matrix residual");
    static_assert(GRAD || !FORCES, "forces come with the adjoint");
    static_assert(!COMP || (!FORCES && NS > 1), "the centre-image path has no forces and several sites");
    static_assert(!BOUND || (!GRAD && !COMP && !CHARGED), "the error scale is for uncharged forward grids");
    static_assert(!STATS || (!GRAD && !BOUND), "the work counts are for forward passes");
    constexpr bool COLS = (GRAD && !FORCES) || BOUND;
    const int tid = threadIdx.x;
    const bool valid = io.valid;
    const long long item = io.item;

    // ---- guest site positions, 32-bit fixed-point fractions of the supercell ----
    uint32_t ux[NS], uy[NS], uz[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) ux[k] = uy[k] = uz[k] = 0u;
    uint32_t cfix[3] = {0u, 0u, 0u};  // the pose centre (COMP)
    bool blocked = false;  // inaccessible pocket: U = +Inf without its pair terms mattering
    if (valid) {
        if (io.pose_mode == POSE_PHILOX && io.at_point) {
            pose_sites<NS>(S, io.seed, static_cast<unsigned long long>(item + io.item_base), ux, uy, uz, nullptr, cfix,
                           io.com_at);
        } else if (io.pose_mode == POSE_PHILOX) {
            float com[3];
            pose_sites<NS>(S, io.seed, static_cast<unsigned long long>(item), ux, uy, uz, com, cfix);
            if (S.acc) blocked = !accessible_com(S, com);
        } else if (io.pose_mode == POSE_SITES) {
            const uint32_t* p = io.site_fix + static_cast<size_t>(item) * S.n_sites * 3;
#pragma unroll
            for (int k = 0; k < NS; ++k)
                if (k < S.n_sites) {
                    ux[k] = p[3 * k + 0];
                    uy[k] = p[3 * k + 1];
                    uz[k] = p[3 * k + 2];
                }
        } else {
            const long long n1 = io.n1, n2 = io.n2;
            ux[0] = io.grid_x[static_cast<int>(item % n1)];
            uy[0] = io.grid_y[static_cast<int>((item / n1) % n2)];
            uz[0] = io.grid_z[static_cast<int>(item / (n1 * n2))];
        }
    }

    // ---- stream the framework through the TMA ring -------------------------
    const int n_tiles = S.n_tiles, n_rec = S.n_rec, n_seg = S.n_seg;
    const int4* rec = S.rec;
    const SegDesc* segs = S.seg;
    const SitePar* segpar = S.segpar;
    int last_issued = -1;
    auto issue = [&](int t) {
        const int slot = t % PMGB_NSTAGE;
        const int t0 = t * PMGB_TILE;
        const int cnt = min(PMGB_TILE, n_rec - t0);
        const uint32_t bytes = static_cast<uint32_t>(cnt) * sizeof(int4);
        mbar_expect_tx(&bars[slot], bytes);
        bulk_g2s(stage + size_t(slot) * PMGB_TILE, rec + t0, bytes, &bars[slot]);
        last_issued = t;
    };
    if (tid == 0 && !io.resident) {
        fence_proxy_async_smem();  // a previous unit's generic reads of the ring come first
        const int n0 = min(PMGB_NSTAGE, n_tiles);
        for (int t = 0; t < n0; ++t) issue(t);
    }
    const Geo g{S.h00, S.h01, S.h02, S.h11, S.h12, S.h22, S.p00, S.p01, S.p02, S.p11, S.p12, S.p22,
                S.rc2, S.rc2e, S.alpha};
    const Geo2 g2{f2(S.h00), f2(S.h01), f2(S.h02), f2(S.h11), f2(S.h12), f2(S.h22),
                  f2(S.p00), f2(S.p01), f2(S.p02), f2(S.p11), f2(S.p12), f2(S.p22),
                  S.rc2, S.rc2e, fmaxf(S.rc2, CHARGED ? S.rc2e : 0.0f), f2(0.5f * S.alpha),
                  f2(-S.alpha * S.alpha * 1.4426950408889634f)};
    const float2 c1 = f2(1.1283791670955126f * S.alpha);  // 2 alpha / sqrt(pi)
    float qcoul[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) qcoul[k] = S.q[k] * static_cast<float>(S.coul);
    // per-site compensated accumulators (sites past n_sites are placeholders)
    float lj_hi[NS], lj_lo[NS], ph_hi[NS], ph_lo[NS];
    float2 gx[NS], gy[NS], gz[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        lj_hi[k] = lj_lo[k] = ph_hi[k] = ph_lo[k] = 0.0f;
        gx[k] = gy[k] = gz[k] = f2(0.0f);
    }
    bool ovl = false, abort = false;
    int fail_tile = 0;
    unsigned long long st_dist = 0, st_lj = 0, st_es = 0;  // STATS: this item's counts
    // STATS: count the distances of n records to one site and the pairs inside each cutoff
    auto count_pairs = [&](int n, float a, float b, float c, float d) {
        if (STATS && valid && !blocked) {
            st_dist += n;
            st_lj += (a < g2.rc2) + (n > 1 && b < g2.rc2) + (n > 2 && c < g2.rc2) + (n > 3 && d < g2.rc2);
            if (CHARGED)
                st_es += (a < g2.rc2e) + (n > 1 && b < g2.rc2e) + (n > 2 && c < g2.rc2e) + (n > 3 && d < g2.rc2e);
        }
    };
    // BOUND: smallest |r^2 - rc^2| seen, an overlap distance within rounding, sum of squared terms
    float cgap = __int_as_float(0x7f800000);
    bool thr_near = false;
    float bsq = 0.0f, bsum = 0.0f;  // FP32: an estimate (an overflow to +Inf only asks for re-evaluation)
    int cb = 0;  // running sub-chunk index: the order of S.cbox
    const bool box_cull = io.cull && S.cbox != nullptr;

    // ---- centre-image path (COMP) -----------------------------------------------
    // Every image of a record within the cutoff of a site has all its fractional displacements
    // inside (-1/2, 1/2) (the cutoff is below half of every perpendicular width W_d), so it is the
    // site's wrapped image, the only one that can contribute.  Where every W_d >= 2 (cutoff +
    // com_reach) (S.com_axis == -1), that image's displacement from the pose centre lies within
    // cutoff + com_reach < W_d / 2 along every face normal, so it is the centre's wrapped image;
    // and a site whose wrapped image differs lies at least W_d / 2 - com_reach >= cutoff away in
    // both, where every term is an exact zero.  So the records' displacements from the centre are
    // converted once per record and each site subtracts its Cartesian offset: the site registers
    // hold the negated offsets (FP32 bits) from here on, after the reciprocal space has used them
    // as fixed points.
    float plc_hi = 0.0f, plc_lo = 0.0f;
    if constexpr (COMP) {
        if (CHARGED && valid) kspace_fwd<NS, false>(S, ux, uy, uz, plc_hi, plc_lo);
#pragma unroll
        for (int k = 0; k < NS; ++k) {
            float nx = 0.0f, ny = 0.0f, nz = 0.0f;
            if (valid && k < S.n_sites) {
                const float fx = __int2float_rn(static_cast<int>(ux[k] - cfix[0]));
                const float fy = __int2float_rn(static_cast<int>(uy[k] - cfix[1]));
                const float fz = __int2float_rn(static_cast<int>(uz[k] - cfix[2]));
                nx = -(fmaf(g.h00, fx, fmaf(g.h01, fy, g.h02 * fz)) + fmaf(g.p00, fx, fmaf(g.p01, fy, g.p02 * fz)));
                ny = -(fmaf(g.h11, fy, g.h12 * fz) + fmaf(g.p11, fy, g.p12 * fz));
                nz = -fmaf(g.h22, fz, g.p22 * fz);
            }
            ux[k] = __float_as_uint(nx);
            uy[k] = __float_as_uint(ny);
            uz[k] = __float_as_uint(nz);
        }
    }

    for (int t = 0; t < n_tiles; ++t) {
        const int slot = t % PMGB_NSTAGE;
        const uint32_t parity = (fills[slot] + static_cast<uint32_t>(t / PMGB_NSTAGE)) & 1u;
        const bool ok = io.resident || mbar_wait_bounded(&bars[slot], parity);
        if (__syncthreads_or(!ok)) {
            abort = true;
            fail_tile = t;
            break;
        }
        const int4* T = stage + size_t(slot) * PMGB_TILE;
        const int t0 = t * PMGB_TILE;
        const int t1 = min(t0 + PMGB_TILE, n_rec);
        for (int sg = 0; sg < n_seg; ++sg) {
            const SegDesc d = segs[sg];
            const int lo = max(d.lo, t0), hi = min(d.hi, t1);
            if (lo >= hi) continue;
            float sig2[NS], eps4[NS], r2o[NS], segmin[NS], lj12[NS], lj6[NS];
#pragma unroll
            for (int k = 0; k < NS; ++k) {
                const SitePar p = segpar[sg * PMGB_MAX_SITES + k];
                sig2[k] = p.sig2;
                eps4[k] = p.eps4;
                r2o[k] = p.r2ovl;
                lj12[k] = p.lj12;
                lj6[k] = p.lj6;
                segmin[k] = __int_as_float(0x7f800000);
            }
            float2 i12[NS], i6[NS], i24[NS];
#pragma unroll
            for (int k = 0; k < NS; ++k) i12[k] = i6[k] = i24[k] = f2(0.0f);
            for (int j0 = lo; j0 < hi; j0 += kChunk) {
                const int j1 = min(j0 + kChunk, hi);
                const int n_sub = (j1 - j0 + kSub - 1) / kSub;
                // spatially ordered warp: bit s set if some lane may reach a record of sub-chunk s;
                // the others are skipped whole, distances included (warp-uniform)
                unsigned near_sub = (1u << n_sub) - 1u;
                if (box_cull) {
                    if constexpr (COMP) {
                        for (int sb = 0; sb < n_sub; ++sb)
                            if (!chunk_near_com(S, S.cbox + cb + sb, cfix, valid && !blocked)) near_sub &= ~(1u << sb);
                    } else {
                        for (int sb = 0; sb < n_sub; ++sb)
                            if (!chunk_near<NS>(S, S.cbox + cb + sb, ux, uy, uz, valid && !blocked, g2.rcmax2))
                                near_sub &= ~(1u << sb);
                    }
                    cb += n_sub;
                    if (near_sub == 0u) continue;
                }
                float2 ljp2[NS], php2[NS];
#pragma unroll
                for (int k = 0; k < NS; ++k) ljp2[k] = php2[k] = f2(0.0f);
                float ljp[NS], php[NS];
                // the terms of a group of four records after every site's distances: one vote per pair
                // of records (bit 0: some lane reaches records 0-1, bit 1: records 2-3; the terms of a
                // pair no lane reaches are exact zeros); both pairs together where both are reached,
                // for 2 NS independent chains
                auto terms_by_pair = [&](float m01, float m23, const float2 (&d01)[NS], const float2 (&d23)[NS],
                                         const int4& r0, const int4& r1, const int4& r2, const int4& r3) {
                    const bool act = valid && !blocked;
                    // (uncharged: the LJ terms are cheap, one vote for the group costs less)
                    const unsigned flags =
                        CHARGED ? __reduce_or_sync(0xffffffffu,
                                                   act ? (unsigned(m01 < g2.rcmax2) | unsigned(m23 < g2.rcmax2) << 1) : 0u)
                                : (__any_sync(0xffffffffu, act && fminf(m01, m23) < g2.rcmax2) ? 3u : 0u);
                    if (flags == 3u) {
#pragma unroll
                        for (int k = 0; k < NS; ++k) {
                            const float2 a12 = f2(lj12[k]), a6 = f2(lj6[k]);
                            pair2_energy<CHARGED, COLS>(d01[k], __int_as_float(r0.w), __int_as_float(r1.w), g2, a12, a6,
                                                        ljp2[k], php2[k], &i12[k], &i6[k], BOUND ? &i24[k] : nullptr);
                            pair2_energy<CHARGED, COLS>(d23[k], __int_as_float(r2.w), __int_as_float(r3.w), g2, a12, a6,
                                                        ljp2[k], php2[k], &i12[k], &i6[k], BOUND ? &i24[k] : nullptr);
                        }
                    } else if (flags != 0u) {
                        const bool first = flags == 1u;
                        const float qa = __int_as_float(first ? r0.w : r2.w), qb = __int_as_float(first ? r1.w : r3.w);
#pragma unroll
                        for (int k = 0; k < NS; ++k) {
                            const float2 a12 = f2(lj12[k]), a6 = f2(lj6[k]);
                            pair2_energy<CHARGED, COLS>(first ? d01[k] : d23[k], qa, qb, g2, a12, a6, ljp2[k], php2[k],
                                                        &i12[k], &i6[k], BOUND ? &i24[k] : nullptr);
                        }
                    }
                };
                // groups of four over the near sub-chunks, in the order of one sweep over [j0, j1);
                // a skipped last sub-chunk takes the remainder with it.  Returns the first record
                // left (fewer than four).
                auto sweep = [&](auto&& group) {
                    int j = j0;
                    if (near_sub == (1u << n_sub) - 1u) {
                        for (; j + 4 <= j1; j += 4) group(j);
                    } else {
                        for (int sb = 0; sb < n_sub; ++sb) {
                            const int s_end = min(j0 + (sb + 1) * kSub, j1);
                            if (!(near_sub >> sb & 1u)) {
                                j = (sb == n_sub - 1) ? j1 : s_end;
                                continue;
                            }
                            for (; j + 4 <= s_end; j += 4) group(j);
                        }
                    }
                    return j;
                };
                if constexpr (COMP) {
                    // centre images (culled or not: the same arithmetic and order, so culling
                    // changes no sum).  The records' displacements keep the box-matrix residual
                    // in every variant: one conversion per record serves all sites, and that form
                    // gives the single-system and the batch kernels the same roundings.
                    auto group4c = [&](int j) {
                        const int4 r0 = T[j - t0], r1 = T[j + 1 - t0], r2 = T[j + 2 - t0], r3 = T[j + 3 - t0];
                        float2 X01, Y01, Z01, X23, Y23, Z23;
                        com_disp2(r0, r1, cfix[0], cfix[1], cfix[2], g2, X01, Y01, Z01);
                        com_disp2(r2, r3, cfix[0], cfix[1], cfix[2], g2, X23, Y23, Z23);
                        // every site's distances, one vote for the group, then every site's terms
                        float2 d01[NS], d23[NS];
                        float m01 = __int_as_float(0x7f800000), m23 = m01;
#pragma unroll
                        for (int k = 0; k < NS; ++k) {
                            const float nx = __uint_as_float(ux[k]), ny = __uint_as_float(uy[k]),
                                        nz = __uint_as_float(uz[k]);
                            d01[k] = site_r2(X01, Y01, Z01, nx, ny, nz);
                            d23[k] = site_r2(X23, Y23, Z23, nx, ny, nz);
                            segmin[k] = fminf(segmin[k], fminf(fminf(d01[k].x, d01[k].y), fminf(d23[k].x, d23[k].y)));
                            if (k < S.n_sites) {
                                m01 = fminf(m01, fminf(d01[k].x, d01[k].y));
                                m23 = fminf(m23, fminf(d23[k].x, d23[k].y));
                            }
                            count_pairs(4, d01[k].x, d01[k].y, d23[k].x, d23[k].y);
                        }
                        terms_by_pair(m01, m23, d01, d23, r0, r1, r2, r3);
                    };
                    int j = sweep(group4c);
                    for (; j < j1; ++j) {
                        // one record: the second lane of the packed terms is far beyond every
                        // cutoff with no charge, so its terms are exact zeros
                        const int4 r = T[j - t0];
                        float2 X, Y, Z;
                        com_disp2(r, r, cfix[0], cfix[1], cfix[2], g2, X, Y, Z);
#pragma unroll
                        for (int k = 0; k < NS; ++k) {
                            float2 dd = site_r2(X, Y, Z, __uint_as_float(ux[k]), __uint_as_float(uy[k]),
                                                __uint_as_float(uz[k]));
                            dd.y = 1e30f;
                            segmin[k] = fminf(segmin[k], dd.x);
                            count_pairs(1, dd.x, 0.0f, 0.0f, 0.0f);
                            pair2_energy<CHARGED, COLS>(dd, __int_as_float(r.w), 0.0f, g2, f2(lj12[k]), f2(lj6[k]),
                                                        ljp2[k], php2[k], &i12[k], &i6[k]);
                        }
                    }
#pragma unroll
                    for (int k = 0; k < NS; ++k) {
                        ljp[k] = ljp2[k].x + ljp2[k].y;
                        php[k] = php2[k].x + php2[k].y;
                    }
                } else if (FORCES) {
                    for (int sb = 0; sb < n_sub; ++sb) {
                    if (!(near_sub >> sb & 1u)) continue;
                    const int s_end = min(j0 + (sb + 1) * kSub, j1);
                    for (int j = j0 + sb * kSub; j < s_end; j += 2) {
                        const bool two = j + 1 < j1;
                        const int4 ra = T[j - t0];
                        const int4 rb = two ? T[j + 1 - t0] : ra;
                        const float2 mask = make_float2(1.0f, two ? 1.0f : 0.0f);
#pragma unroll
                        for (int k = 0; k < NS; ++k) {
                            if (io.cull) {
                                // no lane has the site within the cutoff of either record: every
                                // term below would be an exact zero (no overlap is possible either)
                                const float2 d = pair2_r2(ra, rb, ux[k], uy[k], uz[k], g2);
                                if (!__any_sync(0xffffffffu, valid && !blocked && fminf(d.x, d.y) < g2.rcmax2)) continue;
                            }
                            Grad2 G{i12[k], i6[k], gx[k], gy[k], gz[k]};
                            pair2_grad<CHARGED>(ra, rb, ux[k], uy[k], uz[k], g2, f2(lj12[k]), f2(lj6[k]),
                                                f2(qcoul[k]), c1, mask, segmin[k], ljp2[k], php2[k], G);
                            i12[k] = G.i12;
                            i6[k] = G.i6;
                            gx[k] = G.gx;
                            gy[k] = G.gy;
                            gz[k] = G.gz;
                        }
                    }
                    }
#pragma unroll
                    for (int k = 0; k < NS; ++k) {
                        ljp[k] = ljp2[k].x + ljp2[k].y;
                        php[k] = php2[k].x + php2[k].y;
                    }
                } else if (io.cull || BOUND) {
                    // the warp's insertions are spatially close: after the distances, skip the
                    // pair terms of four records when no lane has the site inside the cutoff
                    // (those terms are exact zeros, so the sums are unchanged)
                    auto group4 = [&](int j) {
                        const int4 r0 = T[j - t0], r1 = T[j + 1 - t0], r2 = T[j + 2 - t0], r3 = T[j + 3 - t0];
                        // the distances of every site first, one vote for the group, then the terms of
                        // every site: 2 NS independent chains for the schedulers (the sites of a guest
                        // are near or far together; a far pair's terms are exact zeros either way)
                        float2 d01[NS], d23[NS];
                        float m01 = __int_as_float(0x7f800000), m23 = m01;
#pragma unroll
                        for (int k = 0; k < NS; ++k) {
                            d01[k] = pair2_r2<RESID>(r0, r1, ux[k], uy[k], uz[k], g2);
                            d23[k] = pair2_r2<RESID>(r2, r3, ux[k], uy[k], uz[k], g2);
                            segmin[k] = fminf(segmin[k], fminf(fminf(d01[k].x, d01[k].y), fminf(d23[k].x, d23[k].y)));
                            if (k < S.n_sites) {
                                m01 = fminf(m01, fminf(d01[k].x, d01[k].y));
                                m23 = fminf(m23, fminf(d23[k].x, d23[k].y));
                            }
                            count_pairs(4, d01[k].x, d01[k].y, d23[k].x, d23[k].y);
                            if (BOUND)
                                cgap = fminf(cgap, fminf(fminf(fabsf(d01[k].x - g2.rc2), fabsf(d01[k].y - g2.rc2)),
                                                         fminf(fabsf(d23[k].x - g2.rc2), fabsf(d23[k].y - g2.rc2))));
                        }
                        terms_by_pair(m01, m23, d01, d23, r0, r1, r2, r3);
                    };
                    int j = j0;
                    if (near_sub == (1u << n_sub) - 1u) {
                        for (; j + 4 <= j1; j += 4) group4(j);
                    } else {
                        // sub-chunk by sub-chunk: the same groups of four, in the same order, as one
                        // sweep over [j0, j1); a skipped last sub-chunk takes the remainder with it
                        for (int sb = 0; sb < n_sub; ++sb) {
                            const int s_end = min(j0 + (sb + 1) * kSub, j1);
                            if (!(near_sub >> sb & 1u)) {
                                j = (sb == n_sub - 1) ? j1 : s_end;
                                continue;
                            }
                            for (; j + 4 <= s_end; j += 4) group4(j);
                        }
                    }
#pragma unroll
                    for (int k = 0; k < NS; ++k) {
                        ljp[k] = ljp2[k].x + ljp2[k].y;
                        php[k] = php2[k].x + php2[k].y;
                    }
                    for (; j < j1; ++j) {
                        const int4 r = T[j - t0];
#pragma unroll
                        for (int k = 0; k < NS; ++k) {
                            if (STATS) count_pairs(1, dist2(r, ux[k], uy[k], uz[k], g), 0.0f, 0.0f, 0.0f);
                            pair_fwd<CHARGED, COLS>(r, ux[k], uy[k], uz[k], g, sig2[k], eps4[k], segmin[k], ljp[k],
                                                    php[k], &i12[k].x, &i6[k].x, BOUND ? &i24[k].x : nullptr,
                                                    BOUND ? &cgap : nullptr);
                        }
                    }
                } else {
                    int j = j0;
                    for (; j + 4 <= j1; j += 4) {
                        const int4 r0 = T[j - t0], r1 = T[j + 1 - t0], r2 = T[j + 2 - t0], r3 = T[j + 3 - t0];
#pragma unroll
                        for (int k = 0; k < NS; ++k) {
                            const float2 a12 = f2(lj12[k]), a6 = f2(lj6[k]);
                            pair2_fwd<CHARGED, RESID, COLS>(r0, r1, ux[k], uy[k], uz[k], g2, a12, a6, segmin[k],
                                                            ljp2[k], php2[k], &i12[k], &i6[k]);
                            pair2_fwd<CHARGED, RESID, COLS>(r2, r3, ux[k], uy[k], uz[k], g2, a12, a6, segmin[k],
                                                            ljp2[k], php2[k], &i12[k], &i6[k]);
                        }
                    }
#pragma unroll
                    for (int k = 0; k < NS; ++k) {
                        ljp[k] = ljp2[k].x + ljp2[k].y;
                        php[k] = php2[k].x + php2[k].y;
                    }
                    for (; j < j1; ++j) {
                        const int4 r = T[j - t0];
#pragma unroll
                        for (int k = 0; k < NS; ++k)
                            pair_fwd<CHARGED, COLS>(r, ux[k], uy[k], uz[k], g, sig2[k], eps4[k], segmin[k], ljp[k],
                                                    php[k], &i12[k].x, &i6[k].x);
                    }
                }
#pragma unroll
                for (int k = 0; k < NS; ++k) {
                    two_sum_acc(lj_hi[k], lj_lo[k], ljp[k]);
                    if (CHARGED) two_sum_acc(ph_hi[k], ph_lo[k], php[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < NS; ++k) ovl = ovl || (segmin[k] < r2o[k]);
            if (BOUND) {
                // rep = lj12 r^-12 and att = |lj6| r^-6 per pair inside the cutoff: sum rep^2 + att^2
#pragma unroll
                for (int k = 0; k < NS; ++k) {
                    const float a12 = lj12[k], a6 = lj6[k];
                    const float s12 = i12[k].x + i12[k].y, s6 = i6[k].x + i6[k].y;
                    bsq = fmaf(a12 * a12, i24[k].x + i24[k].y, fmaf(a6 * a6, s12, bsq));
                    bsum = fmaf(a12, s12, fmaf(-a6, s6, bsum));  // lj6 < 0: the attraction's magnitude
                    thr_near = thr_near || fabsf(segmin[k] - r2o[k]) <= 4e-6f * r2o[k];
                }
            }
            if (GRAD && valid) {
                // this thread owns its item's columns: write on the segment's first tile, add after
                const bool first = (lo == d.lo);
#pragma unroll
                for (int k = 0; k < NS; ++k) {
                    float* c12 = io.dsum + static_cast<size_t>((sg * NS + k) * 2) * io.dsum_stride + io.col_item;
                    float* c6 = c12 + io.dsum_stride;
                    const float v12 = i12[k].x + i12[k].y, v6 = i6[k].x + i6[k].y;
                    *c12 = first ? v12 : *c12 + v12;
                    *c6 = first ? v6 : *c6 + v6;
                }
            }
        }
        __syncthreads();  // every thread is done with this slot
        if (tid == 0 && t + PMGB_NSTAGE < n_tiles) {
            fence_proxy_async_smem();
            issue(t + PMGB_NSTAGE);
        }
    }
    if (abort) {
        if (tid == 0) {
            atomicOr(status, PMGB_DEVERR_TMA_TIMEOUT);
            // let copies still in flight land before the CTA's shared memory is released
            for (int t = fail_tile; t <= last_issued; ++t)
                (void)mbar_wait_bounded(&bars[t % PMGB_NSTAGE],
                                        (fills[t % PMGB_NSTAGE] + static_cast<uint32_t>(t / PMGB_NSTAGE)) & 1u);
        }
        return false;
    }
    if (STATS) {  // warp sums, one atomic per counter and warp
        unsigned long long c[3] = {st_dist, st_lj, st_es};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) c[i] += __shfl_xor_sync(0xffffffffu, c[i], o);
            if ((tid & 31) == 0 && c[i]) atomicAdd(io.stats + i, c[i]);
        }
    }
    // every tile t completed one phase of slot t % NSTAGE (none was refilled if resident)
    if (!io.resident) {
#pragma unroll
        for (int s = 0; s < PMGB_NSTAGE; ++s)
            fills[s] += static_cast<uint32_t>(n_tiles > s ? (n_tiles - 1 - s) / PMGB_NSTAGE + 1 : 0);
    }

    // ---- reciprocal space ----------------------------------------------------
    float pl_hi = 0.0f, pl_lo = 0.0f;
    float gu[NS][3];
#pragma unroll
    for (int k = 0; k < NS; ++k) gu[k][0] = gu[k][1] = gu[k][2] = 0.0f;
    if constexpr (COMP) {
        pl_hi = plc_hi;
        pl_lo = plc_lo;
    } else if (CHARGED && valid) {
        kspace_fwd<NS, FORCES>(S, ux, uy, uz, pl_hi, pl_lo, gu);
    }

    // ---- per-item energies (FP64) ----------------------------------------------
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    double uv = 0.0, usr = 0.0, ulr = 0.0;
    float gcx = 0.0f, gcy = 0.0f, gcz = 0.0f;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        if (k < S.n_sites) {
            uv += static_cast<double>(lj_hi[k]) + static_cast<double>(lj_lo[k]);
            if (CHARGED && S.q[k] != 0.0f)
                usr = fma(static_cast<double>(S.q[k]), static_cast<double>(ph_hi[k]) + static_cast<double>(ph_lo[k]), usr);
            if (FORCES) {
                // real space: dU/dx_site = -2 sum c dU/dr^2; reciprocal space: G^T dU/du
                gcx += -2.0f * (gx[k].x + gx[k].y) + S.g00 * gu[k][0];
                gcy += -2.0f * (gy[k].x + gy[k].y) + S.g01 * gu[k][0] + S.g11 * gu[k][1];
                gcz += -2.0f * (gz[k].x + gz[k].y) + S.g02 * gu[k][0] + S.g12 * gu[k][1] + S.g22 * gu[k][2];
            }
        }
    }
    if (ovl) uv = inf;
    usr *= S.coul;
    if (CHARGED) ulr = static_cast<double>(pl_hi) + static_cast<double>(pl_lo);
    if (blocked) {  // src/henry.jl:230-233: energy.vdw = energy.es = Inf
        uv = inf;
        usr = inf;
        ulr = 0.0;
        gcx = gcy = gcz = 0.0f;
    }
    if (FORCES && valid && io.grad_u) {
        io.grad_u[3 * item + 0] = gcx;
        io.grad_u[3 * item + 1] = gcy;
        io.grad_u[3 * item + 2] = gcz;
    }
    if (io.out_mode == OUT_ENERGY) {
        if (valid) {
            io.e_out[3 * item + 0] = uv;
            io.e_out[3 * item + 1] = usr;
            io.e_out[3 * item + 2] = ulr;
        }
        return true;
    }
    if (io.out_mode == OUT_GRID) {
        if (valid) {
            io.grid_out[item] = static_cast<float>(uv * static_cast<double>(io.unit_factor));
            if (GRAD && io.u_out) io.u_out[item] = uv;
            if (BOUND) {
                const bool edge = thr_near || cgap <= 4e-6f * g.rc2;
                const float e = fmaf(2e-8f, bsum, fminf(io.bound_rho * bsum, io.bound_stat * sqrtf(bsq)));
                io.bound_out[item] = (edge || !(e < __int_as_float(0x7f800000))) ? __int_as_float(0x7f800000) : e;
            }
        }
        return true;
    }

    // ---- Widom: log-sum-exp Boltzmann partials of this unit ----------------------
    const double ues = usr + ulr;
    if (valid && io.u_out) {
        io.u_out[2 * item + 0] = uv;
        io.u_out[2 * item + 1] = ues;
    }
    double x = -inf, ev = 0.0, ee = 0.0;
    long long ninf = 0;
    if (valid) {
        const double u = uv + ues;
        if (isfinite(u)) {
            x = -u * io.inv_temperature;
            ev = uv;
            ee = ues;
        } else {
            ninf = 1;
        }
    }
    if (io.x_out) *io.x_out = x;
    if (io.partial) lse_cta(x, ev, ee, ninf, red, io.partial, io.m_out);
    return true;
}

__device__ __forceinline__ void ring_init(uint64_t* bars) {
    if (threadIdx.x == 0) {
#pragma unroll
        for (int s = 0; s < PMGB_NSTAGE; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
}

}  // namespace

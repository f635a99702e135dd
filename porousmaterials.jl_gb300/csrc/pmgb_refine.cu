// pmgb_refine.cu -- FP64 refinement of the Boltzmann tail of a Widom run.
//
// The FP32 pass gives every insertion's energy to ~1e-7 of the sum of its pair-term
// magnitudes.  A block's K_H is a log-sum of e^{-U/T}, so its error is the Boltzmann-weighted
// mean of the per-insertion errors: for frameworks whose weight sits on a few deep sites it
// reaches 1e-6..1e-5 relative.  This pass re-evaluates, in FP64, the insertions that carry
// all but a fraction `tail` of each block's Boltzmann weight and corrects the block sums:
//   1. histogram of the weight e^{x_i - L_b} (x = -U/T, L_b = log of the block sum) over the
//      gap L_b - x_i, in integer fixed point (order-independent, so deterministic);
//   2. per block, the smallest gap cut that leaves at most `tail` of the weight above it;
//   3. stable compaction of the selected insertions (count, scan, scatter in index order);
//   4. high-precision energies of each selected insertion from its exact pose: LJ with the
//      reference's strict cutoff and overlap rule, real-space q erfc(alpha r)/r, and the
//      reciprocal-space sum against S(k) with exact fixed-point phases.  Tiny systems take one
//      thread per insertion in FP64; the others are cut into chunks of records and k-space rows,
//      one warp each, computing in double-float (hi + lo FP32 pairs, ~48 bits) on the FP32 pipes
//      after an FP32 screen queues the pairs near the insertion;
//   5. the refined insertions' FP64 energies replace the FP32 ones in u; the Boltzmann partials of
//      the chunks holding them are formed again from u and their blocks' results recombined.
// The unrefined remainder then contributes at most tail x (its largest FP32 error)/T to
// log K_H.
// The same double-float pass also serves the exact single-configuration energies: entries from
// explicit FP64 coordinates (every configuration) or from screened energy-grid points.
#include "pmgb_device.cuh"

#include <algorithm>

namespace {

constexpr int kBins = 256;             // histogram bins of the gap L - x
constexpr double kBinWidth = 0.25;     // in units of kT: the histogram spans 64 kT
constexpr double kWeightScale = 1099511627776.0;  // 2^40: fixed-point weight (weights sum to 1)

// Where thread `tid` of chunk `cta` sits: its system, statistics block (global index over
// systems x blocks), insertion index within the system and slot in the energy array u.
struct TailRef {
    int sys, gblk;
    long long item, ui;
    bool valid;
};

__device__ __forceinline__ TailRef tail_locate(const RefineArgs& a, int cta, int tid) {
    TailRef t;
    if (a.systems) {
        t.sys = a.chunk_sys[cta];
        const BatchSystem& bs = a.systems[t.sys];
        const int local = cta - bs.chunk_first;
        const int blk = local / bs.ctas_per_block;
        const long long within = static_cast<long long>(local % bs.ctas_per_block) * PMGB_THREADS + tid;
        t.valid = within < bs.n_per_block;
        t.item = static_cast<long long>(blk) * bs.n_per_block + within;
        t.gblk = t.sys * a.n_blocks + blk;
        t.ui = bs.u_base + t.item;
    } else {
        t.sys = 0;
        const int blk = cta / a.ctas_per_block;
        const long long within = static_cast<long long>(cta % a.ctas_per_block) * PMGB_THREADS + tid;
        t.valid = within < a.n_per_block;
        t.item = static_cast<long long>(blk) * a.n_per_block + within;
        t.gblk = blk;
        t.ui = t.item;
    }
    return t;
}

__device__ __forceinline__ double inv_temp(const RefineArgs& a) {
    return a.run ? a.run->inv_temperature : a.inv_temperature;
}

// bin of an insertion (-1: not eligible: infinite energy or empty block)
__device__ __forceinline__ int tail_bin(const RefineArgs& a, const TailRef& t, double* w_out) {
    const double L = a.block_out[4 * t.gblk];
    const double x = -(a.u[2 * t.ui] + a.u[2 * t.ui + 1]) * inv_temp(a);
    if (!isfinite(x) || !isfinite(L)) return -1;
    const double g = fmax(L - x, 0.0);
    if (w_out) *w_out = exp(-g);
    return static_cast<int>(fmin(g * (1.0 / kBinWidth), static_cast<double>(kBins - 1)));
}

__global__ void tail_hist_kernel(const __grid_constant__ RefineArgs a) {
    __shared__ unsigned long long sh[kBins];
    for (int i = threadIdx.x; i < kBins; i += blockDim.x) sh[i] = 0ull;
    __syncthreads();
    const TailRef t = tail_locate(a, blockIdx.x, threadIdx.x);  // one (system, block) per chunk
    if (t.valid) {
        double w = 0.0;
        const int bin = tail_bin(a, t, &w);
        // rounded up: the tail weight is never under-estimated
        const unsigned long long q = (bin >= 0) ? static_cast<unsigned long long>(ceil(w * kWeightScale)) : 0ull;
        if (q) atomicAdd(&sh[bin], q);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kBins; i += blockDim.x)
        if (sh[i]) atomicAdd(&a.hist[static_cast<size_t>(t.gblk) * kBins + i], sh[i]);
}

// cut[g] = number of leading bins to refine: the bins from cut[g] on hold at most tail x total
__global__ void tail_cut_kernel(const __grid_constant__ RefineArgs a) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.n_systems * a.n_blocks) return;
    const unsigned long long* h = a.hist + static_cast<size_t>(g) * kBins;
    double total = 0.0;
    for (int i = 0; i < kBins; ++i) total += static_cast<double>(h[i]);
    const double allowed = a.tail * total;
    double above = 0.0;
    int cut = kBins;
    while (cut > 0 && above + static_cast<double>(h[cut - 1]) <= allowed) {
        above += static_cast<double>(h[cut - 1]);
        --cut;
    }
    a.cut[g] = cut;
}

__device__ __forceinline__ bool selected(const RefineArgs& a, const TailRef& t) {
    if (!t.valid) return false;
    const int bin = tail_bin(a, t, nullptr);
    return bin >= 0 && bin < a.cut[t.gblk];
}

__global__ void tail_count_kernel(const __grid_constant__ RefineArgs a) {
    const TailRef t = tail_locate(a, blockIdx.x, threadIdx.x);
    const int c = __syncthreads_count(selected(a, t) ? 1 : 0);
    if (threadIdx.x == 0) a.counts[blockIdx.x] = c;
}

// exclusive scan of the per-CTA counts (one CTA, sequential over chunks of its size)
__global__ void tail_scan_kernel(const __grid_constant__ RefineArgs a, int n_ctas) {
    __shared__ int sh[1024];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n_ctas; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = (i < n_ctas) ? a.counts[i] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < static_cast<int>(blockDim.x); o <<= 1) {  // Hillis-Steele inclusive scan
            const int t = (static_cast<int>(threadIdx.x) >= o) ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < n_ctas) a.offsets[i] = carry + sh[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += sh[threadIdx.x];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.offsets[n_ctas] = carry;
}

__global__ void tail_scatter_kernel(const __grid_constant__ RefineArgs a) {
    __shared__ int warp_base[PMGB_THREADS / 32];
    const TailRef t = tail_locate(a, blockIdx.x, threadIdx.x);
    const bool sel = selected(a, t);
    const unsigned ballot = __ballot_sync(0xffffffffu, sel);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) warp_base[warp] = __popc(ballot);
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = a.offsets[blockIdx.x];
        for (int w = 0; w < PMGB_THREADS / 32; ++w) {
            const int c = warp_base[w];
            warp_base[w] = acc;
            acc += c;
        }
    }
    __syncthreads();
    if (sel)
        a.list[warp_base[warp] + __popc(ballot & ((1u << lane) - 1u))] =
            (static_cast<long long>(t.sys) << 40) | t.item;
}

// 1/x in FP64 from the FP32 hardware estimate and two Newton steps y <- y + y (1 - x y)
// (quadratic convergence: ~1e-7 -> ~1e-14 -> last-bit accuracy), for x > 0 in FP32 range.
__device__ __forceinline__ double rcp64(double x) {
    double y = static_cast<double>(__frcp_rn(static_cast<float>(x)));
    y = fma(y, fma(-x, y, 1.0), y);
    y = fma(y, fma(-x, y, 1.0), y);
    return y;
}

// erfc(alpha r) / r at s = r^2 from the system's piecewise polynomial table (built on the host
// from the C library's erfc by Chebyshev interpolation at 8 nodes per interval; within ~2e-15 of
// 1/r, i.e. of the bare Coulomb term); pairs closer than 2^-3.5 A use the direct formula.
__device__ __forceinline__ double erfc_over_r(const SysDev& S, double s) {
    const long long bits = __double_as_longlong(s);
    const int oct = static_cast<int>((bits >> 52) & 0x7ff) - 1023 - S.es_e_lo;
    if (oct < 0) {
        const double r = sqrt(s);
        return erfc(S.alpha64 * r) * rcp64(r);
    }
    const int m = static_cast<int>((bits >> 47) & (PMGB_ES_SUB - 1));
    const double x = __longlong_as_double((bits & 0x000fffffffffffffll) | 0x3ff0000000000000ll);  // s 2^-e
    const double t = fma(x, 2.0 * PMGB_ES_SUB, -(2.0 * PMGB_ES_SUB + 1.0 + 2.0 * m));
    const double* c = S.es_tab + PMGB_ES_COEF * (oct * PMGB_ES_SUB + m);
    double v = __ldg(c + PMGB_ES_COEF - 1);
#pragma unroll
    for (int j = PMGB_ES_COEF - 2; j >= 0; --j) v = fma(v, t, __ldg(c + j));
    return v;
}

// Pair terms of one (record, guest site) in FP64: LJ (strict cutoff, overlap flag) and the
// unscaled real-space Coulomb term q_k q_j erfc(alpha r) / r.
__device__ __forceinline__ void pair_fp64(const SysDev& S, int sg, int k, double rx, double ry, double rz, double qj,
                                          const double* x, double& v, double& sr, bool& ovl) {
    double fx = rx - x[0], fy = ry - x[1], fz = rz - x[2];
    fx -= rint(fx);  // nearest image, one shift per axis (Xtals nearest_image!)
    fy -= rint(fy);
    fz -= rint(fz);
    const double cx = S.f2c64[0] * fx + S.f2c64[1] * fy + S.f2c64[2] * fz;
    const double cy = S.f2c64[3] * fy + S.f2c64[4] * fz;
    const double cz = S.f2c64[5] * fz;
    const double r2 = cx * cx + cy * cy + cz * cz;
    const double2 p = S.segpar64[sg * PMGB_MAX_SITES + k];  // (sigma^2, 4 eps); sigma^2 < 0: no LJ
    if (p.x >= 0.0) {
        if (r2 < 0.1) {
            ovl = true;  // R²_OVERLAP, src/vdw_energetics.jl:2,36-37
        } else if (r2 < S.rc2_64) {
            const double t = p.x * rcp64(r2);
            const double t3 = t * t * t;
            v += p.y * (t3 * t3 - t3);
        }
    }
    if (S.charged && qj != 0.0 && S.q64[k] != 0.0 && r2 < S.rc2e_64 && r2 > 0.0)
        sr += S.q64[k] * qj * erfc_over_r(S, r2);
}

// ---- double-float arithmetic (value = hi + lo, two FP32 numbers) ----------------------------
// Error-free sums and products (Knuth's TwoSum, Dekker's Fast2Sum, the FMA product error) written
// with the round-to-nearest intrinsics, which the compiler neither contracts nor reassociates; a
// double-float carries ~48 significant bits and runs on the FP32 pipes (FP64 runs at 1/64 of
// their rate on this GPU).
struct dfl {
    float hi, lo;
};
__device__ __forceinline__ dfl two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ dfl fast_two_sum(float a, float b) {  // |a| >= |b| (or a == 0)
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dfl df_add(dfl x, dfl y) {
    const dfl s = two_sum(x.hi, y.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ dfl df_add_f(dfl x, float y) {
    const dfl s = two_sum(x.hi, y);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, x.lo));
}
__device__ __forceinline__ dfl df_mul(dfl x, dfl y) {
    const float p = __fmul_rn(x.hi, y.hi);
    float e = __fmaf_rn(x.hi, y.hi, -p);
    e = __fmaf_rn(x.hi, y.lo, e);
    e = __fmaf_rn(x.lo, y.hi, e);
    return fast_two_sum(p, e);
}
__device__ __forceinline__ dfl df_sqr(dfl x) {
    const float p = __fmul_rn(x.hi, x.hi);
    float e = __fmaf_rn(x.hi, x.hi, -p);
    e = __fmaf_rn(__fmul_rn(2.0f, x.hi), x.lo, e);
    return fast_two_sum(p, e);
}
// 1/x: the FP32 reciprocal q and one correction q r, r = 1 - x q evaluated in double-float
__device__ __forceinline__ dfl df_rcp(dfl x) {
    const float q = __frcp_rn(x.hi);
    const float p = __fmul_rn(x.hi, q);
    const float pe = __fmaf_rn(x.hi, q, -p);                            // x.hi q = p + pe exactly
    const float r = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, p), pe), __fmul_rn(x.lo, q));
    return fast_two_sum(q, __fmul_rn(r, q));
}
__device__ __forceinline__ bool df_lt(dfl a, float2 b) { return a.hi < b.x || (a.hi == b.x && a.lo < b.y); }
__device__ __forceinline__ dfl df_of(float2 v) { return {v.x, v.y}; }
__device__ __forceinline__ double df_to_double(dfl x) { return static_cast<double>(x.hi) + static_cast<double>(x.lo); }

// erfc(alpha r)/r at s = r^2 (double-float) from the double-float table: interval from the FP32
// bits of s.hi, t = 64 x - (65 + 2 m) exact in its high part; terms t^4.. in FP32 (they are below
// 1e-3 of the value), t^3.. t^0 in double-float.  Outside the table: the FP64 form.
__device__ __forceinline__ dfl erfc_over_r_df(const SysDev& S, dfl s) {
    const uint32_t bits = __float_as_uint(s.hi);
    const int e = static_cast<int>((bits >> 23) & 0xff) - 127;
    const int oct = e - S.es_e_lo;
    if (oct < 0 || oct >= S.es_n_oct) {
        const double v = erfc_over_r(S, df_to_double(s));
        const float hi = static_cast<float>(v);
        return {hi, static_cast<float>(v - static_cast<double>(hi))};
    }
    const int m = static_cast<int>((bits >> 18) & (PMGB_ES_SUB - 1));
    const float xh = __uint_as_float((bits & 0x007fffffu) | 0x3f800000u);          // s.hi 2^-e in [1, 2)
    const float xl = __fmul_rn(s.lo, __uint_as_float(static_cast<uint32_t>(127 - e) << 23));  // s.lo 2^-e
    const float th = __fmaf_rn(xh, 2.0f * PMGB_ES_SUB, -(2.0f * PMGB_ES_SUB + 1.0f + 2.0f * m));  // exact
    const dfl t = fast_two_sum(th, __fmul_rn(xl, 2.0f * PMGB_ES_SUB));
    const float2* c = S.es_tab_df + PMGB_ES_COEF * (oct * PMGB_ES_SUB + m);
    float p = __ldg(c + PMGB_ES_COEF - 1).x;
#pragma unroll
    for (int j = PMGB_ES_COEF - 2; j >= 4; --j) p = fmaf(p, t.hi, __ldg(c + j).x);
    dfl v{p, 0.0f};
#pragma unroll
    for (int j = 3; j >= 0; --j) v = df_add(df_mul(v, t), df_of(__ldg(c + j)));
    return v;
}

// ---- reciprocal space in double-float ------------------------------------------------------
struct dfc {
    dfl re, im;
};
__device__ __forceinline__ dfl df_neg(dfl x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ dfc dfc_mul(dfc a, dfc b) {
    return {df_add(df_mul(a.re, b.re), df_neg(df_mul(a.im, b.im))), df_add(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}

// e^{-2 pi i j / 256}, j < 256, as double-float (re hi, re lo, im hi, im lo): built once per device
// (pmgb_launch_phase_table, at context creation) and copied into each CTA's shared memory, so a
// refinement launch pays no FP64 sincos per CTA.
__device__ float4 g_phase_tab[256];

__global__ void phase_table_kernel() {
    const int j = threadIdx.x;
    if (j >= 256) return;
    double sn, cs;
    sincospi(-static_cast<double>(j) / 128.0, &sn, &cs);
    const float ch = static_cast<float>(cs), sh = static_cast<float>(sn);
    g_phase_tab[j] = make_float4(ch, static_cast<float>(cs - static_cast<double>(ch)), sh,
                                 static_cast<float>(sn - static_cast<double>(sh)));
}

__device__ __forceinline__ void phase_table_init(float4* tab) {
    for (int j = threadIdx.x; j < 256; j += blockDim.x) tab[j] = g_phase_tab[j];
}

// e^{-2 pi i P / 2^64} for a 64-bit fixed-point phase P (exact modulo one turn): the table entry of
// its top 8 bits times e^{-i phi}, phi = 2 pi (the next 48 bits) < 2 pi / 256, by the Taylor
// series of sin and cos (truncation below 1e-19; the terms below 1e-8 of the value in FP32)
__device__ __forceinline__ dfc phase64(uint64_t P, const float4* tab) {
    const float4 t = tab[static_cast<int>(P >> 56)];
    const float rh = __fmul_rn(__uint2float_rn(static_cast<uint32_t>(P >> 32) & 0xffffffu), 2.3283064365386963e-10f);
    const float rl = __fmul_rn(__uint2float_rn(static_cast<uint32_t>(P >> 8) & 0xffffffu), 1.3877787807814457e-17f);
    const dfl phi = df_mul(fast_two_sum(rh, rl), dfl{6.2831854820251465f, -1.7484556e-07f});  // x 2 pi
    const dfl p2 = df_sqr(phi);
    // sin phi = phi (1 - p2/6 + p2^2/120 - p2^3/5040)
    const float ss = __fmul_rn(__fmul_rn(p2.hi, p2.hi), fmaf(p2.hi, -1.0f / 5040.0f, 1.0f / 120.0f));
    const dfl sn = df_mul(phi, df_add_f(df_add(dfl{1.0f, 0.0f}, df_mul(p2, dfl{-0.16666667f, 4.9670538e-09f})), ss));
    // cos phi = 1 - p2/2 + p2^2/24 - p2^3/720 + p2^4/40320
    const dfl c4 = df_mul(df_sqr(p2), dfl{0.041666668f, -1.2417635e-09f});
    const float cs6 = __fmul_rn(__fmul_rn(__fmul_rn(p2.hi, p2.hi), p2.hi), fmaf(p2.hi, 1.0f / 40320.0f, -1.0f / 720.0f));
    const dfl cs = df_add_f(df_add(df_add(dfl{1.0f, 0.0f}, dfl{-0.5f * p2.hi, -0.5f * p2.lo}), c4), cs6);
    return dfc_mul(dfc{dfl{t.x, t.y}, dfl{t.z, t.w}}, dfc{cs, df_neg(sn)});
}

// 64-bit fixed point of a fractional coordinate (x - floor(x)) 2^64, rounded
__device__ __forceinline__ uint64_t frac2fix128(double x) {
    double f = x - floor(x);
    if (f >= 1.0) f = 0.0;
    return __double2ull_rn(f * 18446744073709551616.0);
}

// Reciprocal-space potential of one guest site over the half-rows [row0, row_end) stepping by
// row_step, sum_k Re[wt S(k) e^{-ik.x}], in double-float: row starts from exact 64-bit fixed-point
// phases, steps along kc by the recurrence.  U[d] = ks[d] times the site's fractional coordinate d
// as a 64-bit fixed point (the strides applied in fixed point).
__device__ dfl kspace_df_rows(const SysDev& S, const uint64_t* U, int row0, int row_end, int row_step,
                              const float4* tab) {
    const uint64_t U0 = U[0], U1 = U[1], U2 = U[2];
    const dfc w = phase64(U2, tab);  // one step along +kc
    dfl lr{0.0f, 0.0f};
    for (int row = row0; row < row_end; row += row_step) {
        const KRow R = S.krow[row];
        const uint64_t P = static_cast<uint64_t>(static_cast<int64_t>(R.ka)) * U0 +
                           static_cast<uint64_t>(static_cast<int64_t>(R.kb)) * U1 +
                           static_cast<uint64_t>(static_cast<int64_t>(R.kc0)) * U2;
        dfc e = phase64(P, tab);
        const dfc sw{w.re, R.dir > 0 ? w.im : df_neg(w.im)};  // downward rows step by the conjugate
        const float4* T = S.tk_df + R.off;
        for (int m = 0; m < R.n; ++m) {
            const float4 t = __ldg(T + m);
            lr = df_add(lr, df_add(df_mul(dfl{t.x, t.y}, e.re), df_neg(df_mul(dfl{t.z, t.w}, e.im))));
            e = dfc_mul(e, sw);
        }
    }
    return lr;
}

// FP32 screen of the (record, guest site) pairs.  The guest sites are taken to the records'
// 32-bit fixed point once per insertion; a pair is passed on to pair_fp64 unless its FP32
// distance lies beyond every cutoff plus 0.01 A (the FP32 distance is within ~1e-4 A of the
// FP64 one) -- so the pairs skipped are exactly pairs to which the FP64 path adds nothing, and
// the refined energies do not change.  A pair whose fixed-point difference lies within 2^-12 of
// half a cell on some axis is always passed on: there the two nearest-image choices may differ.
struct SiteScreen {
    uint32_t x[PMGB_MAX_SITES], y[PMGB_MAX_SITES], z[PMGB_MAX_SITES];
    float rx[PMGB_MAX_SITES], ry[PMGB_MAX_SITES], rz[PMGB_MAX_SITES];  // beyond the fixed point (2^-32 units)
    dfl q[PMGB_MAX_SITES];                                              // guest charges
    uint64_t U[PMGB_MAX_SITES][3];  // 64-bit fixed-point fractions times the k-vector strides (reciprocal space)
    float r2max;
};

// FP64 fractional coordinate d of guest site k of entry `item` (supercell fractions):
//  - a Widom insertion: its pose (make_pose) applied to the FP64 site offsets in FP64 (the
//    same products as the FP32 pass's pose_sites, without the rounding to fixed point);
//  - explicit configurations: the caller's FP64 coordinates;
//  - an energy-grid point (single site): (i/(n-1)) / rep per axis, the end plane folded onto
//    the first (its periodic image, as the FP32 grid pass evaluates it).
__device__ __forceinline__ double grid_coord(const RefineArgs& a, unsigned long long point, int d) {
    unsigned long long i;
    if (point < (1ull << 32)) {  // 32-bit division where it suffices
        const unsigned p = static_cast<unsigned>(point), n1 = a.grid_n[0], n2 = a.grid_n[1];
        i = d == 0 ? p % n1 : d == 1 ? (p / n1) % n2 : p / (n1 * n2);
    } else {
        const unsigned long long n1 = a.grid_n[0], n2 = a.grid_n[1];
        i = d == 0 ? point % n1 : d == 1 ? (point / n1) % n2 : point / (n1 * n2);
    }
    // the host's table holds these very FP64 values, (i / (n - 1), minus 1 on the end plane) / rep
    if (a.grid_ax64) return a.grid_ax64[(d > 0 ? a.grid_n[0] : 0) + (d > 1 ? a.grid_n[1] : 0) + i];
    const int n = a.grid_n[d];
    double f = n > 1 ? static_cast<double>(i) / static_cast<double>(n - 1) : 0.0;
    if (f >= 1.0) f -= 1.0;
    return f / static_cast<double>(a.grid_rep[d]);
}

__device__ __forceinline__ double site_coord(const RefineArgs& a, const SysDev& S, unsigned long long seed,
                                             unsigned long long item, int k, int d) {
    if (a.pose_src == REFINE_POSE_SITES) return a.site_xf[(item * S.n_sites + k) * 3 + d];
    if (a.pose_src == REFINE_POSE_GRID) return grid_coord(a, item, d);
    // a Widom pose: its rotation applied to the FP64 site offsets; the centre of mass drawn with
    // it, or (rotational grids) the block's grid point
    const bool at_point = a.pose_src == REFINE_POSE_ROTGRID;
    float xf[3], R[9];
    make_pose(seed, at_point ? item + a.item_base : item, xf, R);
    const double c = at_point ? grid_coord(a, a.point_base + item / a.n_per_block, d) : static_cast<double>(xf[d]);
    const double bx = S.body64[k][0], by = S.body64[k][1], bz = S.body64[k][2];
    const double ox = fma(static_cast<double>(R[0]), bx, fma(static_cast<double>(R[3]), by, static_cast<double>(R[6]) * bz));
    const double oy = fma(static_cast<double>(R[1]), bx, fma(static_cast<double>(R[4]), by, static_cast<double>(R[7]) * bz));
    const double oz = fma(static_cast<double>(R[2]), bx, fma(static_cast<double>(R[5]), by, static_cast<double>(R[8]) * bz));
    if (d == 0) return c + fma(S.g64[0], ox, fma(S.g64[1], oy, S.g64[2] * oz));
    if (d == 1) return c + fma(S.g64[3], oy, S.g64[4] * oz);
    return c + S.g64[5] * oz;
}

// The guest sites of entry `item`, set up once per warp: lane 3k + d (k < n_sites, d < 3) takes
// coordinate d of site k in FP64 (site_coord), then to the 32-bit fixed point with its FP32
// remainder and to the 64-bit fixed-point phase; lane 3k also splits the charge of site k into
// a double-float.  The lanes then exchange the values, so the FP64 set-up costs a warp one pass
// instead of one per site and coordinate.
__device__ __forceinline__ void warp_site_setup(const RefineArgs& a, const SysDev& S, unsigned long long seed,
                                                unsigned long long item, SiteScreen& sc) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int k = min(lane / 3, S.n_sites - 1), d = lane % 3;
    // only the lanes whose values are read below do the FP64 work
    uint32_t fix = 0;
    float rem = 0.0f, qh = 0.0f, ql = 0.0f;
    uint64_t U = 0;
    if (lane < 3 * S.n_sites) {
        const double x = site_coord(a, S, seed, item, k, d);
        const double ux = x * 4294967296.0;
        const long long fx = __double2ll_rn(ux);
        fix = static_cast<uint32_t>(fx);  // as frac2fix64
        rem = static_cast<float>(ux - static_cast<double>(fx));
        U = S.charged ? static_cast<uint64_t>(S.ks[d]) * frac2fix128(x) : 0ull;
        qh = static_cast<float>(S.q64[k]);
        ql = static_cast<float>(S.q64[k] - static_cast<double>(qh));
    }
    for (int kk = 0; kk < S.n_sites; ++kk) {
        const int l = 3 * kk;
        sc.x[kk] = __shfl_sync(full, fix, l);
        sc.y[kk] = __shfl_sync(full, fix, l + 1);
        sc.z[kk] = __shfl_sync(full, fix, l + 2);
        sc.rx[kk] = __shfl_sync(full, rem, l);
        sc.ry[kk] = __shfl_sync(full, rem, l + 1);
        sc.rz[kk] = __shfl_sync(full, rem, l + 2);
        sc.U[kk][0] = __shfl_sync(full, U, l);
        sc.U[kk][1] = __shfl_sync(full, U, l + 1);
        sc.U[kk][2] = __shfl_sync(full, U, l + 2);
        sc.q[kk] = {__shfl_sync(full, qh, l), __shfl_sync(full, ql, l)};
    }
    const float rmax = sqrtf(static_cast<float>(fmax(S.rc2_64, S.charged ? S.rc2e_64 : 0.0))) + 0.01f;
    sc.r2max = rmax * rmax;
}

// The same set-up by one thread from the composed FP64 sites xs (the one-thread-per-insertion
// path; the reciprocal-space phases are not needed there).
__device__ __forceinline__ void screen_init(const SysDev& S, const double (*xs)[3], SiteScreen& sc) {
    for (int k = 0; k < S.n_sites; ++k) {
        const double ux = xs[k][0] * 4294967296.0, uy = xs[k][1] * 4294967296.0, uz = xs[k][2] * 4294967296.0;
        const long long fx = __double2ll_rn(ux), fy = __double2ll_rn(uy), fz = __double2ll_rn(uz);
        sc.x[k] = static_cast<uint32_t>(fx);
        sc.y[k] = static_cast<uint32_t>(fy);
        sc.z[k] = static_cast<uint32_t>(fz);
        sc.rx[k] = static_cast<float>(ux - static_cast<double>(fx));
        sc.ry[k] = static_cast<float>(uy - static_cast<double>(fy));
        sc.rz[k] = static_cast<float>(uz - static_cast<double>(fz));
        const float qh = static_cast<float>(S.q64[k]);
        sc.q[k] = {qh, static_cast<float>(S.q64[k] - static_cast<double>(qh))};
    }
    const float rmax = sqrtf(static_cast<float>(fmax(S.rc2_64, S.charged ? S.rc2e_64 : 0.0))) + 0.01f;
    sc.r2max = rmax * rmax;
}

__device__ __forceinline__ bool near_half_cell(int d) { return d > 0x7FF00000 || d < -0x7FF00000; }

// bit k set: pair (record r, site k) may lie inside a cutoff
__device__ __forceinline__ unsigned screen_pairs(const SysDev& S, const SiteScreen& sc, int4 r) {
    unsigned near = 0;
    for (int k = 0; k < S.n_sites; ++k) {
        const int dx = static_cast<int>(static_cast<uint32_t>(r.x) - sc.x[k]);
        const int dy = static_cast<int>(static_cast<uint32_t>(r.y) - sc.y[k]);
        const int dz = static_cast<int>(static_cast<uint32_t>(r.z) - sc.z[k]);
        const float fx = static_cast<float>(dx), fy = static_cast<float>(dy), fz = static_cast<float>(dz);
        const float cx = fmaf(S.h00, fx, fmaf(S.h01, fy, S.h02 * fz));
        const float cy = fmaf(S.h11, fy, S.h12 * fz);
        const float cz = S.h22 * fz;
        const float r2 = fmaf(cx, cx, fmaf(cy, cy, cz * cz));
        if (r2 <= sc.r2max || near_half_cell(dx) || near_half_cell(dy) || near_half_cell(dz)) near |= 1u << k;
    }
    return near;
}

// Reciprocal-space energy of guest site k over the half-rows [row0, row_end) stepping by
// row_step: Sum_k wt Re[S(k) e^{-ik.x}], the phasor carried along kc by an FP64 recurrence
// from one sincospi per row (rows hold at most a few dozen k-vectors).
__device__ __forceinline__ double kspace_fp64_rows(const SysDev& S, const double* x, int row0, int row_end,
                                                   int row_step) {
    double lr = 0.0;
    double wr, wi;  // e^{-2 pi i ks2 x_c}: one step along +kc
    sincospi(-2.0 * (S.ks[2] * x[2]), &wi, &wr);
    for (int row = row0; row < row_end; row += row_step) {
        const KRow R = S.krow[row];
        double er, ei;  // e^{-ik.x} at the row start (integer products exact)
        sincospi(-2.0 * (static_cast<double>(R.ka * S.ks[0]) * x[0] + static_cast<double>(R.kb * S.ks[1]) * x[1] +
                         static_cast<double>(R.kc0 * S.ks[2]) * x[2]),
                 &ei, &er);
        const double swi = R.dir * wi;  // downward rows step by the conjugate
        const double* sk = S.sk64 + 2 * R.off;
        const double* wt = S.wt64 + R.off;
        for (int m = 0; m < R.n; ++m) {
            lr = fma(wt[m], fma(sk[2 * m], er, -sk[2 * m + 1] * ei), lr);  // Re[S e] with e = er + i ei
            const double nr = fma(er, wr, -ei * swi);
            ei = fma(er, swi, ei * wr);
            er = nr;
        }
    }
    return lr;
}

// FP64 energies of one insertion (guest sites at FP64 fractional coordinates xs), evaluated
// by one thread.
__device__ void energy_fp64_thread(const SysDev& S, const double (*xs)[3], double* out3) {
    const int ns = S.n_sites;
    double v = 0.0, sr = 0.0, lr = 0.0;
    bool ovl = false;
    SiteScreen sc;
    screen_init(S, xs, sc);
    for (int sg = 0; sg < S.n_seg; ++sg) {
        const SegDesc d = S.seg[sg];
        for (int j = d.lo; j < d.hi; ++j) {
            const unsigned near = screen_pairs(S, sc, S.rec[j]);
            if (!near) continue;
            const double qj = S.rec_q[j];
            const double rx = S.rec_xf[3 * j], ry = S.rec_xf[3 * j + 1], rz = S.rec_xf[3 * j + 2];
            for (int k = 0; k < ns; ++k)
                if (near >> k & 1u) pair_fp64(S, sg, k, rx, ry, rz, qj, xs[k], v, sr, ovl);
        }
    }
    if (S.charged)
        for (int k = 0; k < ns; ++k)
            if (S.q64[k] != 0.0) lr += S.q64[k] * kspace_fp64_rows(S, xs[k], 0, S.n_krow, 1);
    out3[0] = ovl ? __longlong_as_double(0x7ff0000000000000ll) : v;
    out3[1] = sr * S.coul;
    out3[2] = lr;
}

// Entries of the per-warp queue of screened pairs: record index << 3 | guest site.
constexpr int kQueueLen = 32 + 32 * PMGB_MAX_SITES;  // a partial round + one batch of 32 records
static_assert(PMGB_MAX_SITES <= 8, "queue entries keep the guest site in 3 bits");

// One queued (record, site) pair in double-float: the displacement from the 32-bit fixed points
// (exact nearest image, as the screen) plus the remainders beyond them, Cartesian through the
// double-float box, then the terms of pair_fp64.
__device__ __forceinline__ dfl fix_disp(uint32_t rf, float rr, uint32_t sf, float sr_) {
    const int i = static_cast<int>(rf - sf);
    const float ih = __int2float_rn(i);
    const dfl di{ih, __int2float_rn(i - __float2int_rn(ih))};  // exact: |i - ih| < 2^8
    return df_add_f(di, __fsub_rn(rr, sr_));
}
__device__ __forceinline__ void queued_pair(const SysDev& S, int sg, int e, const SiteScreen& sc, dfl& v, dfl& sr,
                                            bool& ovl) {
    const int j = e >> 3, k = e & 7;
    const int4 rf = __ldg(S.rec + j);
    const float4 rq = __ldg(S.rec_rq + j);
    const dfl dx = fix_disp(static_cast<uint32_t>(rf.x), rq.x, sc.x[k], sc.rx[k]);
    const dfl dy = fix_disp(static_cast<uint32_t>(rf.y), rq.y, sc.y[k], sc.ry[k]);
    const dfl dz = fix_disp(static_cast<uint32_t>(rf.z), rq.z, sc.z[k], sc.rz[k]);
    const dfl cx = df_add(df_add(df_mul(df_of(S.h_df[0]), dx), df_mul(df_of(S.h_df[1]), dy)), df_mul(df_of(S.h_df[2]), dz));
    const dfl cy = df_add(df_mul(df_of(S.h_df[3]), dy), df_mul(df_of(S.h_df[4]), dz));
    const dfl cz = df_mul(df_of(S.h_df[5]), dz);
    const dfl r2 = df_add(df_add(df_sqr(cx), df_sqr(cy)), df_sqr(cz));
    const float4 p = __ldg(S.segpar_df + sg * PMGB_MAX_SITES + k);  // sigma^2 (hi, lo), 4 eps (hi, lo)
    if (p.x >= 0.0f) {
        if (df_lt(r2, make_float2(0.1f, 1.4901161e-09f))) {  // 0.1 as a double-float (R²_OVERLAP)
            ovl = true;
        } else if (df_lt(r2, S.rc2_df)) {
            const dfl t = df_mul(dfl{p.x, p.y}, df_rcp(r2));
            const dfl t3 = df_mul(df_sqr(t), t);
            const dfl u = df_add(df_sqr(t3), dfl{-t3.hi, -t3.lo});
            v = df_add(v, df_mul(dfl{p.z, p.w}, u));
        }
    }
    if (S.charged && rq.w != 0.0f && sc.q[k].hi != 0.0f && df_lt(r2, S.rc2e_df) && r2.hi > 0.0f) {
        const dfl qq = df_mul(sc.q[k], dfl{rq.w, __ldg(S.rec_qlo + j)});
        sr = df_add(sr, df_mul(qq, erfc_over_r_df(S, r2)));
    }
}

// Part of the FP64 energies evaluated by one warp: framework records [j0, j1) and k-space half-rows
// [k0, k1).  The lanes screen 32 records at a time in FP32 and queue the (record, site) pairs that
// may lie inside a cutoff in `queue` (kQueueLen entries of this warp's shared memory); their terms
// run in double-float in full rounds of 32 queued pairs, so a warp pays only for pairs near the
// insertion however they are spread over its lanes.  k-space half-rows: lanes stride over them.
// The lane sums are added across the warp in double-float.
// out4 = (U_vdw part, U_sr part / coul, U_lr part, overlap).
__device__ void energy_fp64_warp_part(const RefineArgs& a, const SysDev& S, unsigned long long seed,
                                      unsigned long long item, int j0, int j1, int k0, int k1, double* out4,
                                      int* queue, const float4* phase_tab) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int ns = S.n_sites;
    dfl vd{0.0f, 0.0f}, srd{0.0f, 0.0f}, lrd{0.0f, 0.0f};  // this lane's sums (double-float)
    bool ovl = false;
    SiteScreen sc;
    warp_site_setup(a, S, seed, item, sc);
    for (int sg = 0; sg < S.n_seg; ++sg) {
        const SegDesc d = S.seg[sg];
        const int lo = max(d.lo, j0), hi = min(d.hi, j1);
        int queued = 0;  // warp-uniform
        for (int base = lo; base < hi; base += 32) {
            const int j = base + lane;
            const unsigned near = (j < hi) ? screen_pairs(S, sc, S.rec[j]) : 0u;
            const int c = __popc(near);
            int incl = c;  // inclusive prefix of the lanes' pair counts
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(full, incl, o);
                if (lane >= o) incl += t;
            }
            const int total = __shfl_sync(full, incl, 31);
            int pos = queued + incl - c;
            for (unsigned m = near; m; m &= m - 1) queue[pos++] = (j << 3) | (__ffs(m) - 1);
            queued += total;
            __syncwarp();
            int done = 0;
            for (; queued - done >= 32; done += 32) queued_pair(S, sg, queue[done + lane], sc, vd, srd, ovl);
            // carry the partial round to the front of the queue
            const int left = queued - done;
            const int carry = (lane < left) ? queue[done + lane] : 0;
            __syncwarp();
            if (lane < left) queue[lane] = carry;
            __syncwarp();
            queued = left;
        }
        if (lane < queued) queued_pair(S, sg, queue[lane], sc, vd, srd, ovl);
        __syncwarp();  // the queue is free for the next segment
    }
    if (S.charged && k1 > k0) {
        for (int k = 0; k < ns; ++k)
            if (sc.q[k].hi != 0.0f)
                lrd = df_add(lrd, df_mul(sc.q[k], kspace_df_rows(S, sc.U[k], k0 + lane, k1, 32, phase_tab)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        vd = df_add(vd, dfl{__shfl_xor_sync(full, vd.hi, o), __shfl_xor_sync(full, vd.lo, o)});
        srd = df_add(srd, dfl{__shfl_xor_sync(full, srd.hi, o), __shfl_xor_sync(full, srd.lo, o)});
        lrd = df_add(lrd, dfl{__shfl_xor_sync(full, lrd.hi, o), __shfl_xor_sync(full, lrd.lo, o)});
    }
    ovl = __any_sync(full, ovl);
    if (lane == 0) {
        out4[0] = df_to_double(vd);
        out4[1] = df_to_double(srd);
        out4[2] = df_to_double(lrd);
        out4[3] = ovl ? 1.0 : 0.0;
    }
}

// Work units of one insertion (pair terms + reciprocal-space terms).  Tiny insertions are
// evaluated by one thread each; the others are cut into chunks (records and k-space half-rows in
// proportion), one warp per chunk, so that one large insertion spreads over many SMs instead of
// waiting on one warp.  The chunk size adapts to the system's number of refined insertions: ~128
// units (at most 256 chunks) for a single one (a Monte Carlo move: the pass is pure latency, and
// shorter chunks mean shorter chains of dependent loads), ~256 units while its chunk-items stay
// within 256 (a few configurations), ~1024 units while they stay within 4096 (a few insertions: finer
// chunks fill more SMs), else ~16384 units (many insertions: fewer repetitions of the per-chunk
// set-up).  The count is the same for a system alone or in a batch, so the two evaluate identical
// chunks.
__host__ __device__ __forceinline__ long long fp64_work(const SysDev& S) {
    return static_cast<long long>(S.n_sites) * (S.n_rec + (S.charged ? S.n_k : 0));
}
__host__ __device__ __forceinline__ bool small_system(const SysDev& S) { return fp64_work(S) <= 64; }
__host__ __device__ __forceinline__ long long min_ll(long long x, long long y) { return x < y ? x : y; }
__host__ __device__ __forceinline__ int fp64_chunks(const SysDev& S, long long count) {
    if (small_system(S)) return 0;
    if (count == 1) return static_cast<int>(min_ll(256, (fp64_work(S) + 127) / 128));
    const long long finest = min_ll(64, (fp64_work(S) + 255) / 256);
    if (count * finest <= 256) return static_cast<int>(finest);
    const long long fine = min_ll(64, (fp64_work(S) + 1023) / 1024);
    if (count * fine <= 4096) return static_cast<int>(fine);
    return static_cast<int>(min_ll(64, (fp64_work(S) + 16383) / 16384));
}

// The chunk-items of a single-system pass over cnt entries: cnt x fp64_chunks, or one chunk per
// entry when that exceeds the partials' capacity (refine_plan_kernel's rule for one system).
__host__ __device__ __forceinline__ long long single_items(const RefineArgs& a, long long cnt, int* one_chunk) {
    const long long items = cnt * fp64_chunks(a.sys, cnt);
    *one_chunk = items > a.cap_items ? 1 : 0;
    return *one_chunk ? cnt : items;
}

// Pose stream of refined entry e (system << 40 | insertion): its system's seed and insertion index.
__device__ __forceinline__ void entry_pose(const RefineArgs& a, long long e, unsigned long long& seed,
                                           unsigned long long& item) {
    const int sys = static_cast<int>(e >> 40);
    item = static_cast<unsigned long long>(e & ((1ll << 40) - 1));
    seed = a.run ? a.run->seed + static_cast<unsigned long long>(sys) * 0x9E3779B97F4A7C15ull : a.seed;
}

__device__ __forceinline__ void refined_entry(const RefineArgs& a, long long e, const SysDev*& S, double (*xs)[3]) {
    const int sys = static_cast<int>(e >> 40);
    S = a.systems ? &a.systems[sys].sys : &a.sys;
    unsigned long long seed, item;
    entry_pose(a, e, seed, item);
    if (a.pose_src != REFINE_POSE_PHILOX) {
        for (int k = 0; k < S->n_sites; ++k)
            for (int d = 0; d < 3; ++d) xs[k][d] = site_coord(a, *S, seed, item, k, d);
        return;
    }
    // the insertion's pose applied to the FP64 site offsets, kept in FP64 (no fixed point): the
    // products of site_coord with one pose draw for all sites
    float xf[3], R[9];
    make_pose(seed, static_cast<unsigned long long>(item), xf, R);
    for (int k = 0; k < S->n_sites; ++k) {
        const double bx = S->body64[k][0], by = S->body64[k][1], bz = S->body64[k][2];
        const double ox = fma(static_cast<double>(R[0]), bx, fma(static_cast<double>(R[3]), by, static_cast<double>(R[6]) * bz));
        const double oy = fma(static_cast<double>(R[1]), bx, fma(static_cast<double>(R[4]), by, static_cast<double>(R[7]) * bz));
        const double oz = fma(static_cast<double>(R[2]), bx, fma(static_cast<double>(R[5]), by, static_cast<double>(R[8]) * bz));
        xs[k][0] = static_cast<double>(xf[0]) + fma(S->g64[0], ox, fma(S->g64[1], oy, S->g64[2] * oz));
        xs[k][1] = static_cast<double>(xf[1]) + fma(S->g64[3], oy, S->g64[4] * oz);
        xs[k][2] = static_cast<double>(xf[2]) + S->g64[5] * oz;
    }
}

__device__ __forceinline__ const SysDev& entry_system(const RefineArgs& a, long long e) {
    return a.systems ? a.systems[static_cast<int>(e >> 40)].sys : a.sys;
}

// Entries of small systems: one thread each (grid-stride).
__global__ void __launch_bounds__(PMGB_THREADS) refine_small_kernel(const __grid_constant__ RefineArgs a, int n_ctas) {
    const int n_ref = a.offsets[n_ctas];
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_ref; r += gridDim.x * blockDim.x) {
        const long long e = a.list[r];
        if (!small_system(entry_system(a, e))) continue;
        const SysDev* S;
        double xs[PMGB_MAX_SITES][3];
        refined_entry(a, e, S, xs);
        energy_fp64_thread(*S, xs, a.ref_u + 3 * static_cast<size_t>(r));
    }
}

__device__ __forceinline__ int system_entry_first(const RefineArgs& a, int sys) {
    return a.systems ? a.offsets[a.systems[sys].chunk_first] : 0;
}
__device__ __forceinline__ int system_entry_count(const RefineArgs& a, int sys, int n_ctas) {
    if (!a.systems) return a.offsets[n_ctas];
    const BatchSystem& bs = a.systems[sys];
    return a.offsets[bs.chunk_first + bs.ctas_per_block * a.n_blocks] - a.offsets[bs.chunk_first];
}

// plan[s] = first chunk-item of system s (exclusive scan of entries x chunks over systems);
// plan[n_systems] = the total.  If the total would exceed the partials' capacity, every large
// insertion takes one chunk (the total is then at most the number of insertions).
__global__ void __launch_bounds__(1024) refine_plan_kernel(const __grid_constant__ RefineArgs a, int n_ctas) {
    __shared__ long long part[1024];
    __shared__ long long carry;
    __shared__ int one_chunk;
    if (threadIdx.x == 0) {
        carry = 0;
        one_chunk = 0;
        a.counter[0] = 0;
    }
    __syncthreads();
    for (int pass = 0; pass < 2; ++pass) {
        for (int base = 0; base < a.n_systems; base += blockDim.x) {
            const int sys = base + threadIdx.x;
            long long items = 0;
            if (sys < a.n_systems) {
                const SysDev& S = a.systems ? a.systems[sys].sys : a.sys;
                const long long count = system_entry_count(a, sys, n_ctas);
                const int c = fp64_chunks(S, count);
                items = count * (one_chunk && c ? 1 : c);
            }
            part[threadIdx.x] = items;
            __syncthreads();
            for (int o = 1; o < static_cast<int>(blockDim.x); o <<= 1) {
                const long long t = (static_cast<int>(threadIdx.x) >= o) ? part[threadIdx.x - o] : 0;
                __syncthreads();
                part[threadIdx.x] += t;
                __syncthreads();
            }
            if (sys < a.n_systems) a.plan[sys] = static_cast<int>(min(carry + part[threadIdx.x] - items, 0x7fffffffll));
            __syncthreads();
            if (threadIdx.x == blockDim.x - 1) carry += part[threadIdx.x];
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            if (pass == 0 && carry > a.cap_items) {
                one_chunk = 1;  // too many chunk-items for the partials: one chunk per insertion
                carry = 0;
            } else {
                a.plan[a.n_systems] = static_cast<int>(carry);
                a.one_chunk[0] = one_chunk;
            }
        }
        __syncthreads();
        if (!one_chunk || pass == 1) break;
    }
}

// Chunk-items of the large insertions: one warp each, from a work counter.  The warp that
// completes an insertion's last chunk adds the chunk partials in a fixed order (the same sum
// whatever the scheduling) and stores the insertion's FP64 energies.
__global__ void __launch_bounds__(PMGB_THREADS) refine_large_kernel(const __grid_constant__ RefineArgs a, int n_ctas) {
    __shared__ int s_queue[PMGB_THREADS / 32][kQueueLen];
    __shared__ float4 s_phase[256];
    phase_table_init(s_phase);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int total = a.plan[a.n_systems];
    for (;;) {
        int i = 0;
        if (lane == 0) i = atomicAdd(a.counter, 1);
        i = __shfl_sync(0xffffffffu, i, 0);
        if (i >= total || i < 0) break;
        // the system of item i: the last s with plan[s] <= i
        int lo = 0, hi = a.n_systems - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (a.plan[mid] <= i) lo = mid;
            else hi = mid - 1;
        }
        const int sys = lo;
        const SysDev& S = a.systems ? a.systems[sys].sys : a.sys;
        const int C = a.one_chunk[0] ? 1 : fp64_chunks(S, system_entry_count(a, sys, n_ctas));
        const int local = i - a.plan[sys];
        const int r = system_entry_first(a, sys) + local / C;
        const int c = local % C;
        unsigned long long seed, item;
        entry_pose(a, a.list[r], seed, item);
        const int j0 = static_cast<int>(static_cast<long long>(S.n_rec) * c / C);
        const int j1 = static_cast<int>(static_cast<long long>(S.n_rec) * (c + 1) / C);
        const int k0 = static_cast<int>(static_cast<long long>(S.n_krow) * c / C);
        const int k1 = static_cast<int>(static_cast<long long>(S.n_krow) * (c + 1) / C);
        double* p = a.part + 4 * static_cast<size_t>(i);
        energy_fp64_warp_part(a, S, seed, item, j0, j1, k0, k1, p, s_queue[threadIdx.x >> 5], s_phase);
        if (lane == 0 && C == 1) {  // the whole insertion in one chunk
            double* out = a.ref_u + 3 * static_cast<size_t>(r);
            out[0] = p[3] > 0.0 ? __longlong_as_double(0x7ff0000000000000ll) : p[0];
            out[1] = p[1] * S.coul;
            out[2] = p[2];
        } else if (C > 1) {
            int last = 0;
            if (lane == 0) {
                __threadfence();  // this chunk's partial before the count
                last = atomicAdd(&a.done[r], 1) == C - 1;
            }
            if (__shfl_sync(0xffffffffu, last, 0)) {
                // the warp that completes the entry adds the chunk partials: lane l takes chunks
                // l, l + 32, ... in order, then a fixed butterfly over the lanes -- the same sum
                // whatever the scheduling, with loads in flight on every lane instead of a chain
                __threadfence();  // every other chunk's partial is visible
                const double* q = a.part + 4 * static_cast<size_t>(i - c);
                double v = 0.0, sr = 0.0, lr = 0.0, ov = 0.0;
                for (int cc = lane; cc < C; cc += 32) {
                    v += __ldcg(q + 4 * cc);
                    sr += __ldcg(q + 4 * cc + 1);
                    lr += __ldcg(q + 4 * cc + 2);
                    ov += __ldcg(q + 4 * cc + 3);
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    v += __shfl_xor_sync(0xffffffffu, v, o);
                    sr += __shfl_xor_sync(0xffffffffu, sr, o);
                    lr += __shfl_xor_sync(0xffffffffu, lr, o);
                    ov += __shfl_xor_sync(0xffffffffu, ov, o);
                }
                if (lane == 0) {
                    double* out = a.ref_u + 3 * static_cast<size_t>(r);
                    out[0] = ov > 0.0 ? __longlong_as_double(0x7ff0000000000000ll) : v;
                    out[1] = sr * S.coul;
                    out[2] = lr;
                }
            }
        }
    }
}

// The refined insertions' FP64 energies replace the FP32 ones in u (every block, grid-stride).
__global__ void tail_store_kernel(const __grid_constant__ RefineArgs a, int n_ctas) {
    const int n_ref = a.offsets[n_ctas];
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_ref; r += gridDim.x * blockDim.x) {
        const long long e = a.list[r];
        const long long base = a.systems ? a.systems[static_cast<int>(e >> 40)].u_base : 0;
        const long long ui = base + (e & ((1ll << 40) - 1));
        const double* f = a.ref_u + 3 * static_cast<size_t>(r);
        a.u[2 * ui] = f[0];
        a.u[2 * ui + 1] = f[1] + f[2];
    }
}

// The Boltzmann partial of every chunk that holds refined insertions, formed again from u by the
// FP32 pass's own CTA reduction (lse_cta); the other chunks keep theirs.  Forming the sums from
// the energies, rather than adding FP64 - FP32 differences to them, stays exact where the FP32
// pass erred by many kT (energies of ~1e11 K, where 1e-7 relative is hundreds of kT): there the
// differences would cancel the whole sum.
__global__ void __launch_bounds__(PMGB_THREADS) tail_rechunk_kernel(const __grid_constant__ RefineArgs a) {
    __shared__ LsePartial red[PMGB_THREADS / 32];
    if (a.counts[blockIdx.x] == 0) return;  // uniform over the CTA
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    const TailRef t = tail_locate(a, blockIdx.x, threadIdx.x);
    double x = -inf, ev = 0.0, ee = 0.0;
    long long ninf = 0;
    if (t.valid) {
        const double uv = a.u[2 * t.ui], ue = a.u[2 * t.ui + 1];
        const double u = uv + ue;
        if (isfinite(u)) {
            x = -u * inv_temp(a);
            ev = uv;
            ee = ue;
        } else {
            ninf = 1;
        }
    }
    lse_cta(x, ev, ee, ninf, red, a.partials + blockIdx.x, nullptr);
}

// Per (system, block) with refined insertions: its chunk partials combined in a fixed order, as
// the FP32 pass's block reduction combines them (one warp per block).
__global__ void tail_reblock_kernel(const __grid_constant__ RefineArgs a) {
    const int g = blockIdx.x;
    const int lane = threadIdx.x;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    const unsigned full = 0xffffffffu;
    int c0, cpb;
    if (a.systems) {
        const BatchSystem& bs = a.systems[g / a.n_blocks];
        cpb = bs.ctas_per_block;
        c0 = bs.chunk_first + (g % a.n_blocks) * cpb;
    } else {
        cpb = a.ctas_per_block;
        c0 = g * cpb;
    }
    if (a.offsets[c0 + cpb] == a.offsets[c0]) return;  // no refined insertion: the FP32-pass results stand
    const LsePartial* p = a.partials + c0;
    double m = -inf;
    for (int c = lane; c < cpb; c += 32) m = fmax(m, p[c].m);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(full, m, o));
    double s = 0.0, tv = 0.0, te = 0.0;
    long long n = 0;
    for (int c = lane; c < cpb; c += 32) {
        const LsePartial q = p[c];
        const double f = (m == -inf || q.m == -inf) ? 0.0 : exp(q.m - m);
        s += q.s * f;
        tv += q.tv * f;
        te += q.te * f;
        n += q.n_inf;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(full, s, o);
        tv += __shfl_xor_sync(full, tv, o);
        te += __shfl_xor_sync(full, te, o);
        n += __shfl_xor_sync(full, n, o);
    }
    if (lane == 0) {
        // every insertion of the block overlapping gives -inf and 0/0 means, as the reference's
        double* bo = a.block_out + 4 * g;
        bo[0] = (s > 0.0) ? m + log(s) : -inf;
        bo[1] = tv / s;
        bo[2] = te / s;
        bo[3] = static_cast<double>(n);
    }
}

// ---- exact energies of explicit configurations and of energy-grid points --------------------
// The entry list of the double-float pass when every configuration is evaluated: list[i] = i and
// the entry count in offsets[0] (the refinement kernels then run with zero screen chunks).
// The entry list of an exact pass (every entry, in order) and its count; with `plan` also the
// chunk-item plan of the warp pass, its zeroed work counter and the zeroed chunk counts (what
// refine_plan_kernel and a memset would do, folded into this launch for the single-system pass).
__global__ void exact_list_kernel(const __grid_constant__ RefineArgs a, long long n, const int* n_dev, int plan) {
    const long long cnt = n_dev ? static_cast<long long>(*n_dev) : n;
    for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < cnt;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        a.list[i] = i;
        if (plan) a.done[i] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.offsets[0] = static_cast<int>(cnt);
        if (plan) {
            int one = 0;
            const long long items = single_items(a, cnt, &one);
            a.counter[0] = 0;  // the warp pass's work counter starts from the first chunk-item
            a.plan[0] = 0;
            a.plan[1] = static_cast<int>(min_ll(items, 0x7fffffffll));
            a.one_chunk[0] = one;
        }
    }
}

// A grid point goes to the double-float pass when its FP32 error estimate could exceed its
// tolerance max(1e-5 |U|, 1e-4 K), or is +Inf (a pair at the cutoff or overlap distance).  A point
// that overlaps (U = +Inf) away from the threshold is +Inf whatever the rounding of its terms.
__device__ __forceinline__ bool grid_selected(const float* grid, const float* bound, long long p, long long n,
                                              double inv_unit) {
    if (p >= n) return false;
    const float b = bound[p];
    if (isinf(b)) return true;
    const double u = static_cast<double>(grid[p]) * inv_unit;
    if (!isfinite(u)) return false;
    return static_cast<double>(b) > fmax(1e-5 * fabs(u), 1e-4);
}

__global__ void grid_count_kernel(const __grid_constant__ RefineArgs a, const float* grid, const float* bound,
                                  long long n, double inv_unit) {
    const long long p = static_cast<long long>(blockIdx.x) * PMGB_THREADS + threadIdx.x;
    const int c = __syncthreads_count(grid_selected(grid, bound, p, n, inv_unit) ? 1 : 0);
    if (threadIdx.x == 0) a.counts[blockIdx.x] = c;
}

// stable compaction of the selected points (index order), as tail_scatter_kernel
__global__ void grid_scatter_kernel(const __grid_constant__ RefineArgs a, const float* grid, const float* bound,
                                    long long n, double inv_unit) {
    __shared__ int warp_base[PMGB_THREADS / 32];
    const long long p = static_cast<long long>(blockIdx.x) * PMGB_THREADS + threadIdx.x;
    const bool sel = grid_selected(grid, bound, p, n, inv_unit);
    const unsigned ballot = __ballot_sync(0xffffffffu, sel);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) warp_base[warp] = __popc(ballot);
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = a.offsets[blockIdx.x];
        for (int w = 0; w < PMGB_THREADS / 32; ++w) {
            const int c = warp_base[w];
            warp_base[w] = acc;
            acc += c;
        }
    }
    __syncthreads();
    if (sel) a.list[warp_base[warp] + __popc(ballot & ((1u << lane) - 1u))] = p;
}

// the re-evaluated points' van der Waals energies (+Inf on overlap) into the grid
__global__ void grid_write_kernel(const __grid_constant__ RefineArgs a, float* grid, int n_ctas, double unit) {
    const int n_ref = a.offsets[n_ctas];
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_ref; r += gridDim.x * blockDim.x)
        grid[a.list[r]] = static_cast<float>(a.ref_u[3 * static_cast<size_t>(r)] * unit);
}

}  // namespace

int pmgb_grid_screen_ctas(long long n_points) { return static_cast<int>((n_points + PMGB_THREADS - 1) / PMGB_THREADS); }

cudaError_t pmgb_launch_phase_table(cudaStream_t st) {
    phase_table_kernel<<<1, 256, 0, st>>>();
    return cudaGetLastError();
}

cudaError_t pmgb_launch_exact(const RefineArgs& a, long long n, const int* n_dev, int n_sm, cudaStream_t st) {
    if (!n_dev && n <= 0) return cudaSuccess;
    const long long cap = n_dev ? a.cap_entries : n;
    const int blocks = static_cast<int>(std::max(1ll, std::min((cap + 255) / 256, 4ll * n_sm)));
    // one system: only the thread pass (tiny systems) or only the warp pass runs
    const bool small = small_system(a.sys);
    exact_list_kernel<<<blocks, 256, 0, st>>>(a, n, n_dev, small ? 0 : 1);
    if (small) {
        const int tb = static_cast<int>(std::max(1ll, std::min((cap + PMGB_THREADS - 1) / PMGB_THREADS, 4ll * n_sm)));
        refine_small_kernel<<<tb, PMGB_THREADS, 0, st>>>(a, 0);
        return cudaGetLastError();
    }
    // warps for the chunk-items (8 per CTA), when the count is known here; the work counter
    // spreads them whatever the number of CTAs
    long long ctas = 4ll * n_sm;
    if (!n_dev) {
        int one = 0;
        ctas = std::max(1ll, std::min(ctas, (single_items(a, n, &one) + 7) / 8));
    }
    refine_large_kernel<<<static_cast<int>(ctas), PMGB_THREADS, 0, st>>>(a, 0);
    return cudaGetLastError();
}

cudaError_t pmgb_launch_grid_exact(const RefineArgs& a, const float* bound, float* grid, long long n_points,
                                   double unit_factor, int n_sm, cudaStream_t st) {
    if (n_points <= 0) return cudaSuccess;
    const int n_ctas = pmgb_grid_screen_ctas(n_points);
    const double inv_unit = 1.0 / unit_factor;
    grid_count_kernel<<<n_ctas, PMGB_THREADS, 0, st>>>(a, grid, bound, n_points, inv_unit);
    tail_scan_kernel<<<1, 1024, 0, st>>>(a, n_ctas);
    grid_scatter_kernel<<<n_ctas, PMGB_THREADS, 0, st>>>(a, grid, bound, n_points, inv_unit);
    cudaError_t e = cudaMemsetAsync(a.done, 0, sizeof(int) * static_cast<size_t>(n_points), st);
    if (e != cudaSuccess) return e;
    refine_small_kernel<<<4 * n_sm, PMGB_THREADS, 0, st>>>(a, n_ctas);
    refine_plan_kernel<<<1, 1024, 0, st>>>(a, n_ctas);
    refine_large_kernel<<<4 * n_sm, PMGB_THREADS, 0, st>>>(a, n_ctas);
    grid_write_kernel<<<4 * n_sm, 256, 0, st>>>(a, grid, n_ctas, unit_factor);
    return cudaGetLastError();
}

cudaError_t pmgb_launch_refine(const RefineArgs& a, int n_ctas, int n_sm, cudaStream_t st) {
    if (n_ctas <= 0) return cudaSuccess;
    const int n_g = a.n_systems * a.n_blocks;
    cudaError_t e = cudaMemsetAsync(a.hist, 0, sizeof(unsigned long long) * kBins * n_g, st);
    if (e != cudaSuccess) return e;
    tail_hist_kernel<<<n_ctas, PMGB_THREADS, 0, st>>>(a);
    tail_cut_kernel<<<(n_g + 127) / 128, 128, 0, st>>>(a);
    tail_count_kernel<<<n_ctas, PMGB_THREADS, 0, st>>>(a);
    tail_scan_kernel<<<1, 1024, 0, st>>>(a, n_ctas);
    tail_scatter_kernel<<<n_ctas, PMGB_THREADS, 0, st>>>(a);
    e = cudaMemsetAsync(a.done, 0, sizeof(int) * static_cast<size_t>(a.cap_entries), st);
    if (e != cudaSuccess) return e;
    refine_small_kernel<<<4 * n_sm, PMGB_THREADS, 0, st>>>(a, n_ctas);
    refine_plan_kernel<<<1, 1024, 0, st>>>(a, n_ctas);
    refine_large_kernel<<<4 * n_sm, PMGB_THREADS, 0, st>>>(a, n_ctas);
    tail_store_kernel<<<4 * n_sm, 256, 0, st>>>(a, n_ctas);
    tail_rechunk_kernel<<<n_ctas, PMGB_THREADS, 0, st>>>(a);
    tail_reblock_kernel<<<n_g, 32, 0, st>>>(a);
    return cudaGetLastError();
}

size_t pmgb_refine_hist_words() { return kBins; }

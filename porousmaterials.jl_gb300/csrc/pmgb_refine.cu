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
//   4. FP64 energies of each selected insertion, one CTA each: LJ with the reference's strict
//      cutoff and overlap rule, real-space q erfc(alpha r)/r, and the reciprocal-space sum
//      against the FP64 S(k) with exact fixed-point phases;
//   5. per block, the FP64 minus FP32 differences of e^{x}, U_vdw e^{x} and U_es e^{x}, added
//      in index order to the block results; refined energies replace the FP32 ones in u.
// The unrefined remainder then contributes at most tail x (its largest FP32 error)/T to
// log K_H.
#include "pmgb_device.cuh"

namespace {

constexpr int kBins = 256;             // histogram bins of the gap L - x
constexpr double kBinWidth = 0.25;     // in units of kT: the histogram spans 64 kT
constexpr double kWeightScale = 1099511627776.0;  // 2^40: fixed-point weight (weights sum to 1)

__device__ __forceinline__ bool tail_item(const RefineArgs& a, int cta, int tid, long long& item, int& blk) {
    blk = cta / a.ctas_per_block;
    const long long within = static_cast<long long>(cta % a.ctas_per_block) * PMGB_THREADS + tid;
    item = static_cast<long long>(blk) * a.n_per_block + within;
    return within < a.n_per_block;
}

// bin of insertion `item` (-1: not eligible: infinite energy or empty block)
__device__ __forceinline__ int tail_bin(const RefineArgs& a, long long item, int blk, double* w_out) {
    const double L = a.block_out[4 * blk];
    const double x = -(a.u[2 * item] + a.u[2 * item + 1]) * a.inv_temperature;
    if (!isfinite(x) || !isfinite(L)) return -1;
    const double g = fmax(L - x, 0.0);
    if (w_out) *w_out = exp(-g);
    return static_cast<int>(fmin(g * (1.0 / kBinWidth), static_cast<double>(kBins - 1)));
}

__global__ void tail_hist_kernel(const __grid_constant__ RefineArgs a) {
    __shared__ unsigned long long sh[kBins];
    for (int i = threadIdx.x; i < kBins; i += blockDim.x) sh[i] = 0ull;
    __syncthreads();
    long long item;
    int blk;
    if (tail_item(a, blockIdx.x, threadIdx.x, item, blk)) {
        double w = 0.0;
        const int bin = tail_bin(a, item, blk, &w);
        // rounded up: the tail weight is never under-estimated
        const unsigned long long q = (bin >= 0) ? static_cast<unsigned long long>(ceil(w * kWeightScale)) : 0ull;
        if (q) atomicAdd(&sh[bin], q);
    }
    __syncthreads();
    const int b = blockIdx.x / a.ctas_per_block;
    for (int i = threadIdx.x; i < kBins; i += blockDim.x)
        if (sh[i]) atomicAdd(&a.hist[static_cast<size_t>(b) * kBins + i], sh[i]);
}

// cut[b] = number of leading bins to refine: the bins from cut[b] on hold at most tail x total
__global__ void tail_cut_kernel(const __grid_constant__ RefineArgs a) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= a.n_blocks) return;
    const unsigned long long* h = a.hist + static_cast<size_t>(b) * kBins;
    double total = 0.0;
    for (int i = 0; i < kBins; ++i) total += static_cast<double>(h[i]);
    const double allowed = a.tail * total;
    double above = 0.0;
    int cut = kBins;
    while (cut > 0 && above + static_cast<double>(h[cut - 1]) <= allowed) {
        above += static_cast<double>(h[cut - 1]);
        --cut;
    }
    a.cut[b] = cut;
}

__device__ __forceinline__ bool selected(const RefineArgs& a, int cta, int tid, long long& item) {
    int blk;
    if (!tail_item(a, cta, tid, item, blk)) return false;
    const int bin = tail_bin(a, item, blk, nullptr);
    return bin >= 0 && bin < a.cut[blk];
}

__global__ void tail_count_kernel(const __grid_constant__ RefineArgs a) {
    long long item;
    const int c = __syncthreads_count(selected(a, blockIdx.x, threadIdx.x, item) ? 1 : 0);
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
    long long item;
    const bool sel = selected(a, blockIdx.x, threadIdx.x, item);
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
    if (sel) a.list[warp_base[warp] + __popc(ballot & ((1u << lane) - 1u))] = item;
}

// FP64 energies (U_vdw, U_sr, U_lr) of one insertion whose guest sites are at the FP64
// fractional coordinates xs[k][3], evaluated by the whole CTA from the exact FP64 framework
// coordinates (nearest image by rounding each fractional difference, as Xtals' nearest_image!).
__device__ void energy_fp64(const SysDev& S, const double (*xs)[3], double* out3) {
    __shared__ double red[3][PMGB_THREADS / 32];
    __shared__ int red_ovl;
    const int tid = threadIdx.x;
    if (tid == 0) red_ovl = 0;
    const int ns = S.n_sites;
    double v = 0.0, sr = 0.0, lr = 0.0;
    int ovl = 0;
    for (int sg = 0; sg < S.n_seg; ++sg) {
        const SegDesc d = S.seg[sg];
        for (int j = d.lo + tid; j < d.hi; j += blockDim.x) {
            const double qj = S.rec_q[j];
            const double rx = S.rec_xf[3 * j], ry = S.rec_xf[3 * j + 1], rz = S.rec_xf[3 * j + 2];
            for (int k = 0; k < ns; ++k) {
                double fx = rx - xs[k][0], fy = ry - xs[k][1], fz = rz - xs[k][2];
                fx -= rint(fx);
                fy -= rint(fy);
                fz -= rint(fz);
                const double cx = S.f2c64[0] * fx + S.f2c64[1] * fy + S.f2c64[2] * fz;
                const double cy = S.f2c64[3] * fy + S.f2c64[4] * fz;
                const double cz = S.f2c64[5] * fz;
                const double r2 = cx * cx + cy * cy + cz * cz;
                const double2 p = S.segpar64[sg * PMGB_MAX_SITES + k];  // (sigma^2, 4 eps); sigma^2 < 0: no LJ
                if (p.x >= 0.0) {
                    if (r2 < 0.1) {
                        ovl = 1;  // R²_OVERLAP, src/vdw_energetics.jl:2,36-37
                    } else if (r2 < S.rc2_64) {
                        const double t = p.x / r2;
                        const double t3 = t * t * t;
                        v += p.y * (t3 * t3 - t3);
                    }
                }
                if (S.charged && qj != 0.0 && S.q64[k] != 0.0 && r2 < S.rc2e_64) {
                    const double rr = sqrt(r2);
                    sr += S.q64[k] * qj * erfc(S.alpha64 * rr) / rr;
                }
            }
        }
    }
    if (S.charged) {
        for (int kk = tid; kk < S.n_k; kk += blockDim.x) {
            const double ka = S.kabc[3 * kk], kb = S.kabc[3 * kk + 1], kc = S.kabc[3 * kk + 2];
            const double sre = S.sk64[2 * kk], sim = S.sk64[2 * kk + 1], wt = S.wt64[kk];
            for (int k = 0; k < ns; ++k) {
                if (S.q64[k] == 0.0) continue;
                const double t = ka * xs[k][0] + kb * xs[k][1] + kc * xs[k][2];  // k.x in turns
                double sn, cs;
                sincospi(2.0 * t, &sn, &cs);
                lr += S.q64[k] * wt * (sre * cs + sim * sn);  // Re[S(k) e^{-ik.x}]
            }
        }
    }
    // CTA reduction in a fixed order
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v += __shfl_xor_sync(0xffffffffu, v, o);
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
        lr += __shfl_xor_sync(0xffffffffu, lr, o);
    }
    const int warp = tid >> 5, lane = tid & 31;
    __syncthreads();  // red_ovl initialised
    if (ovl) atomicOr(&red_ovl, 1);
    if (lane == 0) {
        red[0][warp] = v;
        red[1][warp] = sr;
        red[2][warp] = lr;
    }
    __syncthreads();
    if (tid == 0) {
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) {
            a0 += red[0][w];
            a1 += red[1][w];
            a2 += red[2][w];
        }
        out3[0] = red_ovl ? __longlong_as_double(0x7ff0000000000000ll) : a0;
        out3[1] = a1 * S.coul;
        out3[2] = a2;
    }
    __syncthreads();  // red and red_ovl are reused by the next call
}

__global__ void __launch_bounds__(PMGB_THREADS) refine_kernel(const __grid_constant__ RefineArgs a, int n_ctas) {
    const int n_ref = a.offsets[n_ctas];
    for (int r = blockIdx.x; r < n_ref; r += gridDim.x) {
        const long long item = a.list[r];
        // the insertion's pose applied to the FP64 site offsets, kept in FP64 (no fixed point)
        float xf[3], R[9];
        make_pose(a.seed, static_cast<unsigned long long>(item), xf, R);
        __shared__ double xs[PMGB_MAX_SITES][3];
        if (threadIdx.x < PMGB_MAX_SITES) {
            const SysDev& S = a.sys;
            const int k = threadIdx.x;
            const double bx = S.body64[k][0], by = S.body64[k][1], bz = S.body64[k][2];
            const double ox = static_cast<double>(R[0]) * bx + static_cast<double>(R[3]) * by + static_cast<double>(R[6]) * bz;
            const double oy = static_cast<double>(R[1]) * bx + static_cast<double>(R[4]) * by + static_cast<double>(R[7]) * bz;
            const double oz = static_cast<double>(R[2]) * bx + static_cast<double>(R[5]) * by + static_cast<double>(R[8]) * bz;
            xs[k][0] = static_cast<double>(xf[0]) + (S.g64[0] * ox + S.g64[1] * oy + S.g64[2] * oz);
            xs[k][1] = static_cast<double>(xf[1]) + (S.g64[3] * oy + S.g64[4] * oz);
            xs[k][2] = static_cast<double>(xf[2]) + S.g64[5] * oz;
        }
        __syncthreads();
        energy_fp64(a.sys, xs, a.ref_u + 3 * static_cast<size_t>(r));  // ends with a barrier
    }
}

// Per block: add the FP64 - FP32 differences of the refined insertions (index order) to the
// block results and store the refined energies in u.
__global__ void tail_correct_kernel(const __grid_constant__ RefineArgs a) {
    const int b = blockIdx.x;
    const int lane = threadIdx.x;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    const int r0 = a.offsets[b * a.ctas_per_block], r1 = a.offsets[(b + 1) * a.ctas_per_block];
    double* bo = a.block_out + 4 * b;
    const double L = bo[0];
    double ds = 0.0, dv = 0.0, de = 0.0;
    long long dn = 0;
    for (int r = r0 + lane; r < r1; r += 32) {
        const long long item = a.list[r];
        const double uv32 = a.u[2 * item], ue32 = a.u[2 * item + 1];
        const double* f = a.ref_u + 3 * static_cast<size_t>(r);
        const double uv64 = f[0], ue64 = f[1] + f[2];
        const double x32 = -(uv32 + ue32) * a.inv_temperature;
        const double x64 = -(uv64 + ue64) * a.inv_temperature;
        const double w32 = exp(x32 - L);
        if (isfinite(x64)) {
            const double w64 = w32 * exp(x64 - x32);
            ds += w32 * expm1(x64 - x32);
            dv += uv64 * w64 - uv32 * w32;
            de += ue64 * w64 - ue32 * w32;
        } else {
            ds -= w32;
            dv -= uv32 * w32;
            de -= ue32 * w32;
            dn += 1;
        }
        a.u[2 * item] = uv64;
        a.u[2 * item + 1] = ue64;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ds += __shfl_xor_sync(0xffffffffu, ds, o);
        dv += __shfl_xor_sync(0xffffffffu, dv, o);
        de += __shfl_xor_sync(0xffffffffu, de, o);
        dn += __shfl_xor_sync(0xffffffffu, dn, o);
    }
    if (lane == 0 && r1 > r0) {
        // block_out = (L, <U_vdw>, <U_es>, n_inf) with sums relative to e^L equal to (1, <U_vdw>, <U_es>)
        const double s = 1.0 + ds;
        if (s > 0.0) {
            bo[0] = L + log1p(ds);
            bo[1] = (bo[1] + dv) / s;
            bo[2] = (bo[2] + de) / s;
        } else {
            // every insertion of the block overlaps: the weighted means are 0/0, as the reference's
            const double nan = __longlong_as_double(0x7ff8000000000000ll);
            bo[0] = -inf;
            bo[1] = nan;
            bo[2] = nan;
        }
        bo[3] += static_cast<double>(dn);
    }
}

}  // namespace

cudaError_t pmgb_launch_refine(const RefineArgs& a, int n_ctas, int n_sm, cudaStream_t st) {
    if (n_ctas <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(a.hist, 0, sizeof(unsigned long long) * kBins * a.n_blocks, st);
    if (e != cudaSuccess) return e;
    tail_hist_kernel<<<n_ctas, PMGB_THREADS, 0, st>>>(a);
    tail_cut_kernel<<<(a.n_blocks + 31) / 32, 32, 0, st>>>(a);
    tail_count_kernel<<<n_ctas, PMGB_THREADS, 0, st>>>(a);
    tail_scan_kernel<<<1, 1024, 0, st>>>(a, n_ctas);
    tail_scatter_kernel<<<n_ctas, PMGB_THREADS, 0, st>>>(a);
    refine_kernel<<<4 * n_sm, PMGB_THREADS, 0, st>>>(a, n_ctas);
    tail_correct_kernel<<<a.n_blocks, 32, 0, st>>>(a);
    return cudaGetLastError();
}

size_t pmgb_refine_hist_words() { return kBins; }

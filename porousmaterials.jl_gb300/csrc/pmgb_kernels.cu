// pmgb_kernels.cu -- single-system sm_103a kernels for the Widom-insertion / energy-grid
// path (one CTA per unit of PMGB_THREADS items), the FP64 reductions behind them, and the
// exported launchers.  The per-unit device body lives in pmgb_device.cuh.
#include "pmgb_device.cuh"

#include <atomic>

namespace {

// Single-system launch: CTA b runs unit b.
template <int NS, bool CHARGED, bool GRAD, bool RESID = true, bool FORCES = GRAD, bool COMP = false,
          bool BOUND = false, bool STATS = false>
__global__ void __launch_bounds__(PMGB_THREADS, 2) pairs_kernel(const __grid_constant__ LaunchArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    int4* stage = reinterpret_cast<int4*>(smem_raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + size_t(PMGB_NSTAGE) * PMGB_TILE * sizeof(int4));
    __shared__ LsePartial red[PMGB_THREADS / 32];
    const int tid = threadIdx.x;
    UnitIO io{};
    io.pose_mode = a.pose_mode;
    io.out_mode = a.out_mode;
    if (a.pose_mode == POSE_PHILOX) {
        const int b = blockIdx.x / a.ctas_per_block;
        const long long slot = static_cast<long long>(blockIdx.x % a.ctas_per_block) * PMGB_THREADS + tid;
        io.valid = slot < a.n_per_block;
        long long within = slot;
        if (a.perm && io.valid) within = a.perm[static_cast<size_t>(b) * a.n_per_block + slot];
        io.item = static_cast<long long>(b) * a.n_per_block + within;
        io.cull = a.perm != nullptr;
        if (a.rot_grid) {
            const long long p = a.point_base + b;
            const long long n1 = a.n_pts[0], n2 = a.n_pts[1];
            io.at_point = true;
            io.com_at[0] = a.grid_x[static_cast<int>(p % n1)];
            io.com_at[1] = a.grid_y[static_cast<int>((p / n1) % n2)];
            io.com_at[2] = a.grid_z[static_cast<int>(p / (n1 * n2))];
            io.item_base = a.item_base;
            io.cull = true;  // every lane of the CTA sits at the same point: skip what none reaches
        }
    } else if (a.pose_mode == POSE_SITES) {
        io.item = static_cast<long long>(blockIdx.x) * PMGB_THREADS + tid;
        io.valid = io.item < a.n_conf;
    } else if (a.grid_bricks) {
        // warp w takes brick (bi, bj, bk) of 4 x 4 x 2 points; i fastest inside it
        const int n1 = a.n_pts[0], n2 = a.n_pts[1], n3 = a.n_pts[2];
        const long long B1 = (n1 + 3) / 4, B2 = (n2 + 3) / 4;
        const long long w = static_cast<long long>(blockIdx.x) * (PMGB_THREADS / 32) + (tid >> 5);
        const int lane = tid & 31;
        const int i = static_cast<int>(w % B1) * 4 + (lane & 3);
        const int j = static_cast<int>((w / B1) % B2) * 4 + ((lane >> 2) & 3);
        const long long k = (w / (B1 * B2)) * 2 + (lane >> 4);
        io.valid = i < n1 && j < n2 && k < n3;
        io.item = io.valid ? i + static_cast<long long>(n1) * (j + static_cast<long long>(n2) * k) : 0;
        io.cull = true;
    } else {
        io.item = static_cast<long long>(blockIdx.x) * PMGB_THREADS + tid;
        io.valid = io.item < static_cast<long long>(a.n_pts[0]) * a.n_pts[1] * a.n_pts[2];
    }
    io.seed = a.seed;
    io.inv_temperature = a.inv_temperature;
    io.site_fix = a.site_fix;
    io.grid_x = a.grid_x;
    io.grid_y = a.grid_y;
    io.grid_z = a.grid_z;
    io.n1 = a.n_pts[0];
    io.n2 = a.n_pts[1];
    io.u_out = a.u_out;
    io.e_out = a.e_out;
    io.grid_out = a.grid_out;
    io.unit_factor = a.unit_factor;
    io.dsum = a.dsum;
    io.dsum_stride = a.dsum_stride;
    io.col_item = io.item;
    io.grad_u = a.grad_u;
    io.bound_out = a.bound_out;
    io.bound_rho = a.bound_rho;
    io.bound_stat = a.bound_stat;
    io.stats = a.stats;
    io.partial = (a.partials && !a.perm) ? a.partials + blockIdx.x : nullptr;
    ring_init(bars);
    uint32_t fills[PMGB_NSTAGE] = {};
    (void)run_unit<NS, CHARGED, GRAD, RESID, FORCES, COMP, BOUND, STATS>(a.sys, io, stage, bars, red, fills,
                                                                          a.status);
}

// ---- latency path: few configurations, one CTA each -----------------------------------
// For Monte Carlo moves (one molecule per call, src/gcmc.jl:111-124 -> vdw_energy): the CTA's
// threads split the framework records (and the k-space half-rows) of one configuration and
// the partial sums meet in a fixed-order FP64 reduction.  Same FP32 pair terms as the Widom
// kernel's scalar path; n_conf comes from device memory when n_conf_dev is set (a captured
// graph serves any count up to its CTA count).
template <int NS, bool CHARGED>
__global__ void __launch_bounds__(PMGB_THREADS) energies_latency_kernel(const __grid_constant__ LaunchArgs a) {
    __shared__ double red[3][PMGB_THREADS / 32];
    __shared__ int red_ovl;
    const SysDev& S = a.sys;
    const long long n_conf = a.n_conf_dev ? static_cast<long long>(*a.n_conf_dev) : a.n_conf;
    const int c = blockIdx.x;
    if (c >= n_conf) return;  // uniform over the CTA
    const int tid = threadIdx.x;
    if (tid == 0) red_ovl = 0;
    uint32_t ux[NS], uy[NS], uz[NS];
    const uint32_t* p = a.site_fix + static_cast<size_t>(c) * S.n_sites * 3;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        ux[k] = k < S.n_sites ? p[3 * k] : 0u;
        uy[k] = k < S.n_sites ? p[3 * k + 1] : 0u;
        uz[k] = k < S.n_sites ? p[3 * k + 2] : 0u;
    }
    const Geo g{S.h00, S.h01, S.h02, S.h11, S.h12, S.h22, S.p00, S.p01, S.p02, S.p11, S.p12, S.p22,
                S.rc2, S.rc2e, S.alpha};
    float lj[NS], ph[NS];
    bool ovl = false;
#pragma unroll
    for (int k = 0; k < NS; ++k) lj[k] = ph[k] = 0.0f;
    for (int sg = 0; sg < S.n_seg; ++sg) {
        const SegDesc d = S.seg[sg];
        float sig2[NS], eps4[NS], r2o[NS], segmin[NS];
#pragma unroll
        for (int k = 0; k < NS; ++k) {
            const SitePar sp = S.segpar[sg * PMGB_MAX_SITES + k];
            sig2[k] = sp.sig2;
            eps4[k] = sp.eps4;
            r2o[k] = sp.r2ovl;
            segmin[k] = __int_as_float(0x7f800000);
        }
        for (int j = d.lo + tid; j < d.hi; j += blockDim.x) {
            const int4 r = __ldg(S.rec + j);
#pragma unroll
            for (int k = 0; k < NS; ++k)
                pair_fwd<CHARGED>(r, ux[k], uy[k], uz[k], g, sig2[k], eps4[k], segmin[k], lj[k], ph[k]);
        }
#pragma unroll
        for (int k = 0; k < NS; ++k) ovl = ovl || (segmin[k] < r2o[k]);
    }
    double v = 0.0, sr = 0.0, lr = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        if (k < S.n_sites) {
            v += static_cast<double>(lj[k]);
            if (CHARGED) sr += static_cast<double>(S.q[k]) * static_cast<double>(ph[k]);
        }
    }
    if (CHARGED) {
        float hi = 0.0f, lo = 0.0f;
        kspace_fwd<NS>(S, ux, uy, uz, hi, lo, nullptr, tid, blockDim.x);
        lr = static_cast<double>(hi) + static_cast<double>(lo);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v += __shfl_xor_sync(0xffffffffu, v, o);
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
        lr += __shfl_xor_sync(0xffffffffu, lr, o);
    }
    __syncthreads();  // red_ovl initialised
    if (ovl) atomicOr(&red_ovl, 1);
    const int warp = tid >> 5, lane = tid & 31;
    if (lane == 0) {
        red[0][warp] = v;
        red[1][warp] = sr;
        red[2][warp] = lr;
    }
    __syncthreads();
    if (tid == 0) {
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        for (int w = 0; w < PMGB_THREADS / 32; ++w) {
            a0 += red[0][w];
            a1 += red[1][w];
            a2 += red[2][w];
        }
        a.e_out[3 * c + 0] = red_ovl ? __longlong_as_double(0x7ff0000000000000ll) : a0;
        a.e_out[3 * c + 1] = a1 * S.coul;
        a.e_out[3 * c + 2] = a2;
    }
}

template <bool CH>
cudaError_t launch_latency_ns(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    switch (a.sys.n_sites <= 1 ? 1 : a.sys.n_sites <= 2 ? 2 : a.sys.n_sites <= 3 ? 3 : a.sys.n_sites <= 4 ? 4
                                                                : a.sys.n_sites <= 6 ? 6 : 8) {
        case 1: energies_latency_kernel<1, CH><<<n_ctas, PMGB_THREADS, 0, st>>>(a); break;
        case 2: energies_latency_kernel<2, CH><<<n_ctas, PMGB_THREADS, 0, st>>>(a); break;
        case 3: energies_latency_kernel<3, CH><<<n_ctas, PMGB_THREADS, 0, st>>>(a); break;
        case 4: energies_latency_kernel<4, CH><<<n_ctas, PMGB_THREADS, 0, st>>>(a); break;
        case 6: energies_latency_kernel<6, CH><<<n_ctas, PMGB_THREADS, 0, st>>>(a); break;
        default: energies_latency_kernel<8, CH><<<n_ctas, PMGB_THREADS, 0, st>>>(a); break;
    }
    return cudaGetLastError();
}

// ---- spatial processing order of a Widom run ----------------------------------------
constexpr int kOrderBits = 5;                       // 32 cells per axis
constexpr int kOrderCells = 1 << (3 * kOrderBits);  // 32768 cells

// Hilbert-curve cell of insertion idx: the top 5 bits of each coordinate of its centre of mass
// (the first Philox draw of make_pose)
__device__ __forceinline__ int widom_cell(unsigned long long seed, unsigned long long idx) {
    const uint2 key = make_uint2(static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    const uint4 a = philox4x32_10(make_uint4(static_cast<uint32_t>(idx), static_cast<uint32_t>(idx >> 32), 0u, 0u), key);
    return hilbert_cell(a.x >> (32 - kOrderBits), a.y >> (32 - kOrderBits), a.z >> (32 - kOrderBits), kOrderBits);
}

__global__ void order_count_kernel(unsigned long long seed, long long n_per_block, long long n, int* counts) {
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long b = i / n_per_block;
    atomicAdd(&counts[b * kOrderCells + widom_cell(seed, static_cast<unsigned long long>(i))], 1);
}

// exclusive scan of one block's 32768 cell counts (1024 threads x 32 consecutive cells)
__global__ void __launch_bounds__(1024) order_scan_kernel(int* counts) {
    __shared__ int part[1024];
    int* c = counts + static_cast<size_t>(blockIdx.x) * kOrderCells;
    constexpr int per = kOrderCells / 1024;
    const int t = threadIdx.x;
    int v[per], sum = 0;
#pragma unroll
    for (int q = 0; q < per; ++q) {
        v[q] = c[t * per + q];
        sum += v[q];
    }
    part[t] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int add = (t >= o) ? part[t - o] : 0;
        __syncthreads();
        part[t] += add;
        __syncthreads();
    }
    int run = part[t] - sum;
#pragma unroll
    for (int q = 0; q < per; ++q) {
        c[t * per + q] = run;
        run += v[q];
    }
}

// Insertions go to their cell's next slot; the order inside a cell is whatever the atomics give,
// which changes nothing: each insertion's energy does not depend on its slot, and the block
// sums are formed afterwards in insertion order.
__global__ void order_scatter_kernel(unsigned long long seed, long long n_per_block, long long n, int* offsets,
                                     int* perm) {
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long b = i / n_per_block;
    const int pos = atomicAdd(&offsets[b * kOrderCells + widom_cell(seed, static_cast<unsigned long long>(i))], 1);
    perm[b * n_per_block + pos] = static_cast<int>(i - b * n_per_block);
}

__global__ void __launch_bounds__(PMGB_THREADS) lse_from_u_kernel(const double* __restrict__ u, long long n_per_block,
                                                                 int ctas_per_block, double inv_t,
                                                                 LsePartial* __restrict__ partials) {
    __shared__ LsePartial red[PMGB_THREADS / 32];
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    const int b = blockIdx.x / ctas_per_block;
    const long long within = static_cast<long long>(blockIdx.x % ctas_per_block) * PMGB_THREADS + threadIdx.x;
    double x = -inf, ev = 0.0, ee = 0.0;
    long long ninf = 0;
    if (within < n_per_block) {
        const long long item = static_cast<long long>(b) * n_per_block + within;
        const double uv = u[2 * item], ues = u[2 * item + 1];
        const double uu = uv + ues;
        if (isfinite(uu)) {
            x = -uu * inv_t;
            ev = uv;
            ee = ues;
        } else {
            ninf = 1;
        }
    }
    lse_cta(x, ev, ee, ninf, red, partials + blockIdx.x, nullptr);
}

// log_scale[0] = max_i (-U_i / T) over finite U (one CTA, fixed order)
__global__ void max_neg_u_kernel(const double* __restrict__ u, long long n, double inv_t, double* __restrict__ out) {
    __shared__ double red[32];
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    double m = -inf;
    for (long long i = threadIdx.x; i < n; i += blockDim.x)
        if (isfinite(u[i])) m = fmax(m, -u[i] * inv_t);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = -inf;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v = fmax(v, red[w]);
        out[0] = v;
    }
}

// Per-chunk weighted column sums: partials[chunk * (n_cols + 2) + c] = sum_{i in chunk} w_i col_c[i],
// with two extra columns sum w_i and sum w_i U_es,i.  w_i = exp(-(U_vdw + U_es)/T - M) where M is
// the largest log-sum of the statistics blocks (so every w_i <= 1), 0 for infinite energies.
__global__ void weighted_columns_kernel(const double* __restrict__ u, int u_stride, long long n, double inv_t,
                                        const double* __restrict__ log_scale, int n_log,
                                        const float* __restrict__ cols, int n_cols, long long col_stride,
                                        double* __restrict__ partials) {
    __shared__ double red[8][34];
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    double M = -inf;
    for (int b = 0; b < n_log; ++b) M = fmax(M, log_scale[4 * b]);
    const long long chunk = (n + gridDim.x - 1) / gridDim.x;
    const long long i0 = blockIdx.x * chunk, i1 = min(n, i0 + chunk);
    const int nc = n_cols + 2;
    for (int c0 = 0; c0 < nc; c0 += 32) {
        double acc[32];
#pragma unroll
        for (int c = 0; c < 32; ++c) acc[c] = 0.0;
        for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
            double ue = 0.0, uu = inf;
            if (u_stride == 2) {
                ue = u[2 * i + 1];
                uu = u[2 * i] + ue;
            } else {
                uu = u[i];
            }
            const double w = (isfinite(uu) && M > -inf) ? exp(-uu * inv_t - M) : 0.0;
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                const int cc = c0 + c;
                // w = 0 for U = +Inf, whose columns may hold Inf: skip rather than form 0 * Inf
                if (cc < n_cols) {
                    if (w > 0.0) acc[c] = fma(w, static_cast<double>(cols[static_cast<size_t>(cc) * col_stride + i]), acc[c]);
                }
                else if (cc == n_cols) acc[c] += w;
                else if (cc == n_cols + 1) acc[c] = fma(w, isfinite(uu) ? ue : 0.0, acc[c]);
            }
        }
        // block reduction in a fixed order
#pragma unroll
        for (int c = 0; c < 32; ++c) {
            double v = acc[c];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][c] = v;
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            double v = 0.0;
            for (int wv = 0; wv < (int)(blockDim.x >> 5); ++wv) v += red[wv][threadIdx.x];
            const int cc = c0 + threadIdx.x;
            if (cc < nc) partials[static_cast<size_t>(blockIdx.x) * nc + cc] = v;
        }
        __syncthreads();
    }
}

__global__ void sum_partials_kernel(const double* __restrict__ partials, int n_chunks, int nc,
                                    double* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    double v = 0.0;
    for (int k = 0; k < n_chunks; ++k) v += partials[static_cast<size_t>(k) * nc + c];
    out[c] = v;
}

// Combine the per-CTA partials of each statistics block in a fixed order.
// block_out[4b..4b+3] = (log sum e^{-U/T}, <U_vdw>_bf, <U_es>_bf, #insertions with U=+Inf)
__global__ void reduce_blocks_kernel(const LsePartial* __restrict__ partials, int ctas_per_block,
                                     double* __restrict__ block_out) {
    const int b = blockIdx.x;
    const int lane = threadIdx.x;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    const unsigned full = 0xffffffffu;
    const LsePartial* p = partials + static_cast<size_t>(b) * ctas_per_block;
    double m = -inf;
    for (int c = lane; c < ctas_per_block; c += 32) m = fmax(m, p[c].m);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(full, m, o));
    double s = 0.0, tv = 0.0, te = 0.0;
    long long n = 0;
    for (int c = lane; c < ctas_per_block; c += 32) {
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
        block_out[4 * b + 0] = (s > 0.0) ? m + log(s) : -inf;
        block_out[4 * b + 1] = tv / s;
        block_out[4 * b + 2] = te / s;
        block_out[4 * b + 3] = static_cast<double>(n);
    }
}

// Phasor tables for S(k): table[(off_d + h + kmax_d) n_q + c] = e^{2 pi i h x_{c,d}} for each axis
// d and |h| <= kmax_d, one FP64 sincospi each from the exact FP64 charge positions.
__global__ void phasor_table_kernel(const double* __restrict__ qxf, int n_q, int3 kmax, double2* __restrict__ table,
                                    long long n) {
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = static_cast<int>(i % n_q);
    int row = static_cast<int>(i / n_q), d = 0, h;
    const int w0 = 2 * kmax.x + 1, w1 = 2 * kmax.y + 1;
    if (row < w0) {
        h = row - kmax.x;
    } else if (row < w0 + w1) {
        d = 1;
        h = row - w0 - kmax.y;
    } else {
        d = 2;
        h = row - w0 - w1 - kmax.z;
    }
    double sn, cs;
    sincospi(2.0 * static_cast<double>(h) * qxf[3 * c + d], &sn, &cs);
    table[i] = make_double2(cs, sn);
}

// S(k) = sum_c q_c e^{2 pi i (ka fa + kb fb + kc fc)}, the phasor of each charge the product of its
// three axis phasors; one warp per k-vector, lanes over charges, FP64 accumulation.
__global__ void structure_factor_kernel(const double* __restrict__ q, int n_q, const int* __restrict__ kabc,
                                        const double* __restrict__ wt, int n_k, int3 kmax,
                                        const double2* __restrict__ table, double* __restrict__ sk_out,
                                        float2* __restrict__ skw_out) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n_k) return;
    const int w0 = 2 * kmax.x + 1, w1 = 2 * kmax.y + 1;
    const double2* ta = table + static_cast<size_t>(kabc[3 * warp] + kmax.x) * n_q;
    const double2* tb = table + static_cast<size_t>(w0 + kabc[3 * warp + 1] + kmax.y) * n_q;
    const double2* tc = table + static_cast<size_t>(w0 + w1 + kabc[3 * warp + 2] + kmax.z) * n_q;
    double re = 0.0, im = 0.0;
    for (int c = lane; c < n_q; c += 32) {
        const double2 a = ta[c], b = tb[c], e = tc[c];
        const double abr = fma(a.x, b.x, -a.y * b.y), abi = fma(a.x, b.y, a.y * b.x);
        const double pr = fma(abr, e.x, -abi * e.y), pi = fma(abr, e.y, abi * e.x);
        re = fma(q[c], pr, re);
        im = fma(q[c], pi, im);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == 0) {
        sk_out[2 * warp] = re;
        sk_out[2 * warp + 1] = im;
        skw_out[warp] = make_float2(static_cast<float>(wt[warp] * re), static_cast<float>(wt[warp] * im));
    }
}

__global__ void sample_poses_kernel(unsigned long long seed, long long start, long long n, float* xf_out,
                                    float* rot_out) {
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float xf[3], R[9];
    make_pose(seed, static_cast<unsigned long long>(start + i), xf, R);
    for (int d = 0; d < 3; ++d) xf_out[3 * i + d] = xf[d];
    for (int d = 0; d < 9; ++d) rot_out[9 * i + d] = R[d];
}

__global__ void philox_kernel(const unsigned int* ctr, const unsigned int* key, long long n, unsigned int* out) {
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint4 r = philox4x32_10(make_uint4(ctr[4 * i], ctr[4 * i + 1], ctr[4 * i + 2], ctr[4 * i + 3]),
                                  make_uint2(key[2 * i], key[2 * i + 1]));
    out[4 * i] = r.x;
    out[4 * i + 1] = r.y;
    out[4 * i + 2] = r.z;
    out[4 * i + 3] = r.w;
}

// Guest-host van der Waals energy in FP64 in the reference's own operation order, one
// configuration per thread (src/vdw_energetics.jl:25-47): for each guest site i (outer) the
// displacements x_j - x_i of the atoms in their given order, Xtals' nearest_image! (d -= sign(d)
// where |d| > 1/2), Cartesian = f_to_c d summed left to right, r^2 = (dx^2 + dy^2) + dz^2, and for
// r^2 < rc^2: +Inf if r^2 < 0.1, else E += ((4 eps) t) (t - 1) with t = (s2 / r^2)^3 = (u u) u.
// Every operation is an explicit round-to-nearest FP64 operation (no contraction into FMAs),
// so configurations whose energies are equal in exact arithmetic compare as the reference's
// FP64 arithmetic compares them.  Serial in the atoms: meant for a handful of configurations.
__global__ void vdw_ordered_kernel(const double* __restrict__ f2c, int n_atoms, const double* __restrict__ atom_xf,
                                   const int* __restrict__ atom_sp, int n_sp, const double* __restrict__ eps,
                                   const double* __restrict__ sig2, double r2_cut, long long n_conf, int n_sites,
                                   const int* __restrict__ site_sp, const double* __restrict__ site_xf,
                                   double* __restrict__ out) {
    const long long c = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= n_conf) return;
    double f[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) f[k] = f2c[k];  // column-major f_to_c: f[i + 3 j] = M[i][j]
    double energy = 0.0;
    for (int i = 0; i < n_sites; ++i) {
        const double* xi = site_xf + (c * n_sites + i) * 3;
        const double x0 = xi[0], x1 = xi[1], x2 = xi[2];
        const int si = site_sp[i];
        for (int j = 0; j < n_atoms; ++j) {
            double d[3] = {__dsub_rn(atom_xf[3 * j], x0), __dsub_rn(atom_xf[3 * j + 1], x1),
                           __dsub_rn(atom_xf[3 * j + 2], x2)};
#pragma unroll
            for (int k = 0; k < 3; ++k)
                if (fabs(d[k]) > 0.5) d[k] = __dsub_rn(d[k], d[k] > 0.0 ? 1.0 : -1.0);
            double r[3];
#pragma unroll
            for (int k = 0; k < 3; ++k)
                r[k] = __dadd_rn(__dadd_rn(__dmul_rn(f[k], d[0]), __dmul_rn(f[k + 3], d[1])), __dmul_rn(f[k + 6], d[2]));
            const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(r[0], r[0]), __dmul_rn(r[1], r[1])), __dmul_rn(r[2], r[2]));
            if (r2 < r2_cut) {
                if (r2 < 0.1) {
                    energy = __longlong_as_double(0x7ff0000000000000LL);  // +Inf, as the reference returns
                    i = n_sites;
                    break;
                }
                const int sj = atom_sp[j];
                const double u = __ddiv_rn(sig2[si * n_sp + sj], r2);
                const double t = __dmul_rn(__dmul_rn(u, u), u);
                energy = __dadd_rn(energy, __dmul_rn(__dmul_rn(__dmul_rn(4.0, eps[si * n_sp + sj]), t),
                                                     __dsub_rn(t, 1.0)));
            }
        }
    }
    out[c] = energy;
}

// FP32 FMA throughput probe: 8 independent dependency chains per thread.
__global__ void __launch_bounds__(256) fp32_peak_kernel(float* sink, int iters) {
    float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
    float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
    const float b = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            a0 = fmaf(a0, b, c); a1 = fmaf(a1, b, c); a2 = fmaf(a2, b, c); a3 = fmaf(a3, b, c);
            a4 = fmaf(a4, b, c); a5 = fmaf(a5, b, c); a6 = fmaf(a6, b, c); a7 = fmaf(a7, b, c);
        }
    }
    const float r = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (r == 12345.678f) sink[blockIdx.x] = r;
}

// the centre-image variant serves Widom poses of guests with several sites where the system's
// geometry allows it (SysDev::com_axis)
__host__ __forceinline__ bool centre_image(const LaunchArgs& a) {
    return a.pose_mode == POSE_PHILOX && a.sys.com_axis >= -1 && a.sys.n_sites > 1;
}

template <int NS, bool CH, bool RESID, bool COMP>
cudaError_t launch_one_rc(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    const size_t smem = pmgb_pairs_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(pairs_kernel<NS, CH, false, RESID, false, COMP>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    pairs_kernel<NS, CH, false, RESID, false, COMP><<<n_ctas, PMGB_THREADS, smem, st>>>(a);
    return cudaGetLastError();
}

// (the centre-image variant keeps the box-matrix residual whether or not refinement follows)
template <int NS, bool CH, bool RESID>
cudaError_t launch_one_r(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    if constexpr (NS > 1)
        if (centre_image(a)) return launch_one_rc<NS, CH, true, true>(a, n_ctas, st);
    return launch_one_rc<NS, CH, RESID, false>(a, n_ctas, st);
}

template <int NS, bool CH>
cudaError_t launch_one(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    return a.no_resid ? launch_one_r<NS, CH, false>(a, n_ctas, st) : launch_one_r<NS, CH, true>(a, n_ctas, st);
}

template <int NS, bool CH, bool FORCES, bool COMP>
cudaError_t launch_grad_one_f(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    const size_t smem = pmgb_pairs_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(pairs_kernel<NS, CH, true, true, FORCES, COMP>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    pairs_kernel<NS, CH, true, true, FORCES, COMP><<<n_ctas, PMGB_THREADS, smem, st>>>(a);
    return cudaGetLastError();
}

// forces (dU/dx) only when the caller asked for them; the columns alone take the forward loops
template <int NS, bool CH>
cudaError_t launch_grad_one(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    if (a.grad_u) return launch_grad_one_f<NS, CH, true, false>(a, n_ctas, st);
    if constexpr (NS > 1)
        if (centre_image(a)) return launch_grad_one_f<NS, CH, false, true>(a, n_ctas, st);
    return launch_grad_one_f<NS, CH, false, false>(a, n_ctas, st);
}

template <bool CH>
cudaError_t launch_grad_ns(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    const int n = a.sys.n_sites;
    if (n <= 1) return launch_grad_one<1, CH>(a, n_ctas, st);
    if (n <= 2) return launch_grad_one<2, CH>(a, n_ctas, st);
    if (n <= 3) return launch_grad_one<3, CH>(a, n_ctas, st);
    if (n <= 4) return launch_grad_one<4, CH>(a, n_ctas, st);
    if (n <= 6) return launch_grad_one<6, CH>(a, n_ctas, st);
    return launch_grad_one<8, CH>(a, n_ctas, st);
}

template <bool CH>
cudaError_t launch_ns(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    const int n = a.sys.n_sites;
    if (n <= 1) return launch_one<1, CH>(a, n_ctas, st);
    if (n <= 2) return launch_one<2, CH>(a, n_ctas, st);
    if (n <= 3) return launch_one<3, CH>(a, n_ctas, st);
    if (n <= 4) return launch_one<4, CH>(a, n_ctas, st);
    if (n <= 6) return launch_one<6, CH>(a, n_ctas, st);
    return launch_one<8, CH>(a, n_ctas, st);
}

}  // namespace

size_t pmgb_pairs_smem_bytes() {
    return size_t(PMGB_NSTAGE) * PMGB_TILE * sizeof(int4) + PMGB_NSTAGE * sizeof(uint64_t);
}

cudaError_t pmgb_launch_pairs(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    if (n_ctas <= 0) return cudaSuccess;
    return a.sys.charged ? launch_ns<true>(a, n_ctas, st) : launch_ns<false>(a, n_ctas, st);
}

cudaError_t pmgb_launch_grid_bound(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    if (n_ctas <= 0) return cudaSuccess;
    if (a.sys.charged || a.sys.n_sites != 1 || a.pose_mode != POSE_GRID || !a.bound_out) return cudaErrorInvalidValue;
    const size_t smem = pmgb_pairs_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(pairs_kernel<1, false, false, true, false, false, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    pairs_kernel<1, false, false, true, false, false, true><<<n_ctas, PMGB_THREADS, smem, st>>>(a);
    return cudaGetLastError();
}

template <int NS, bool CH, bool COMP>
cudaError_t launch_stats_one(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    const size_t smem = pmgb_pairs_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(pairs_kernel<NS, CH, false, true, false, COMP, false, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    pairs_kernel<NS, CH, false, true, false, COMP, false, true><<<n_ctas, PMGB_THREADS, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t pmgb_launch_pairs_stats(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    if (n_ctas <= 0) return cudaSuccess;
    if (!a.stats) return cudaErrorInvalidValue;
    const bool comp = centre_image(a);
    if (a.sys.n_sites == 1)
        return a.sys.charged ? launch_stats_one<1, true, false>(a, n_ctas, st) : launch_stats_one<1, false, false>(a, n_ctas, st);
    if (a.sys.n_sites == 3) {
        if (a.sys.charged)
            return comp ? launch_stats_one<3, true, true>(a, n_ctas, st) : launch_stats_one<3, true, false>(a, n_ctas, st);
        return comp ? launch_stats_one<3, false, true>(a, n_ctas, st) : launch_stats_one<3, false, false>(a, n_ctas, st);
    }
    return cudaErrorNotSupported;
}

cudaError_t pmgb_launch_pairs_grad(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    if (n_ctas <= 0) return cudaSuccess;
    return a.sys.charged ? launch_grad_ns<true>(a, n_ctas, st) : launch_grad_ns<false>(a, n_ctas, st);
}

cudaError_t pmgb_launch_energies_latency(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    if (n_ctas <= 0) return cudaSuccess;
    return a.sys.charged ? launch_latency_ns<true>(a, n_ctas, st) : launch_latency_ns<false>(a, n_ctas, st);
}

size_t pmgb_widom_order_cells() { return kOrderCells; }

cudaError_t pmgb_launch_widom_order(unsigned long long seed, long long n_per_block, int n_blocks, int* counts,
                                    int* perm, cudaStream_t st) {
    const long long n = n_per_block * n_blocks;
    if (n <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * kOrderCells * static_cast<size_t>(n_blocks), st);
    if (e != cudaSuccess) return e;
    const unsigned grid = static_cast<unsigned>((n + 255) / 256);
    order_count_kernel<<<grid, 256, 0, st>>>(seed, n_per_block, n, counts);
    order_scan_kernel<<<n_blocks, 1024, 0, st>>>(counts);
    order_scatter_kernel<<<grid, 256, 0, st>>>(seed, n_per_block, n, counts, perm);
    return cudaGetLastError();
}

cudaError_t pmgb_launch_lse_from_u(const double* u, long long n_per_block, int n_blocks, int ctas_per_block,
                                   double inv_temperature, LsePartial* partials, cudaStream_t st) {
    lse_from_u_kernel<<<n_blocks * ctas_per_block, PMGB_THREADS, 0, st>>>(u, n_per_block, ctas_per_block,
                                                                          inv_temperature, partials);
    return cudaGetLastError();
}

int pmgb_grid_brick_ctas(const int n_pts[3]) {
    const long long bricks = static_cast<long long>((n_pts[0] + 3) / 4) * ((n_pts[1] + 3) / 4) * ((n_pts[2] + 1) / 2);
    return static_cast<int>((bricks + PMGB_THREADS / 32 - 1) / (PMGB_THREADS / 32));
}

cudaError_t pmgb_launch_max_neg_u(const double* u, long long n, double inv_t, double* out, cudaStream_t st) {
    max_neg_u_kernel<<<1, 1024, 0, st>>>(u, n, inv_t, out);
    return cudaGetLastError();
}

cudaError_t pmgb_launch_weighted_columns(const double* u, int u_stride, long long n, double inv_t,
                                         const double* log_scale, int n_log, const float* cols, int n_cols,
                                         long long col_stride, double* partials, int n_chunks, double* out,
                                         cudaStream_t st) {
    weighted_columns_kernel<<<n_chunks, 256, 0, st>>>(u, u_stride, n, inv_t, log_scale, n_log, cols, n_cols,
                                                      col_stride, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int nc = n_cols + 2;
    sum_partials_kernel<<<(nc + 127) / 128, 128, 0, st>>>(partials, n_chunks, nc, out);
    return cudaGetLastError();
}

cudaError_t pmgb_launch_reduce_blocks(const LsePartial* partials, int n_blocks, int ctas_per_block,
                                      double* block_out, cudaStream_t st) {
    reduce_blocks_kernel<<<n_blocks, 32, 0, st>>>(partials, ctas_per_block, block_out);
    return cudaGetLastError();
}

size_t pmgb_structure_factor_table_len(int n_q, const int kmax[3]) {
    return static_cast<size_t>(n_q) * static_cast<size_t>(2 * kmax[0] + 2 * kmax[1] + 2 * kmax[2] + 3);
}

cudaError_t pmgb_launch_structure_factor(const double* qxf, const double* q, int n_q, const int* kabc,
                                         const double* wt, int n_k, const int kmax[3], double2* table,
                                         double* sk_out, float2* skw_out, cudaStream_t st) {
    if (n_k <= 0) return cudaSuccess;
    const int3 km = make_int3(kmax[0], kmax[1], kmax[2]);
    const long long n = static_cast<long long>(pmgb_structure_factor_table_len(n_q, kmax));
    if (n > 0)
        phasor_table_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(qxf, n_q, km, table, n);
    const int warps_per_cta = 8;
    const int ctas = (n_k + warps_per_cta - 1) / warps_per_cta;
    structure_factor_kernel<<<ctas, 32 * warps_per_cta, 0, st>>>(q, n_q, kabc, wt, n_k, km, table, sk_out, skw_out);
    return cudaGetLastError();
}

cudaError_t pmgb_launch_sample_poses(unsigned long long seed, long long start, long long n, float* xf_out,
                                     float* rot_out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    sample_poses_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(seed, start, n, xf_out, rot_out);
    return cudaGetLastError();
}

cudaError_t pmgb_launch_philox(const unsigned int* ctr, const unsigned int* key, long long n, unsigned int* out,
                               cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    philox_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(ctr, key, n, out);
    return cudaGetLastError();
}

cudaError_t pmgb_launch_vdw_ordered(const double* f2c, int n_atoms, const double* atom_xf, const int* atom_sp,
                                    int n_sp, const double* eps, const double* sig2, double r2_cut, long long n_conf,
                                    int n_sites, const int* site_sp, const double* site_xf, double* out,
                                    cudaStream_t st) {
    if (n_conf <= 0) return cudaSuccess;
    vdw_ordered_kernel<<<static_cast<unsigned>((n_conf + 63) / 64), 64, 0, st>>>(
        f2c, n_atoms, atom_xf, atom_sp, n_sp, eps, sig2, r2_cut, n_conf, n_sites, site_sp, site_xf, out);
    return cudaGetLastError();
}

// Self-test of the bounded mbarrier wait the staging ring uses.  One thread initialises an
// mbarrier for one arrival; with `arm` it arrives announcing 16 bytes of transaction that no
// copy will ever deliver (no bulk copy is issued, so nothing is in flight), otherwise it
// arrives plainly and the phase completes.  The wait, limited to limit_ns, then either gives up
// -- the kernel records PMGB_DEVERR_TMA_TIMEOUT in the status word, as the ring's failure path
// does, and returns -- or succeeds.
__global__ void bounded_wait_test_kernel(unsigned int* status, unsigned long long limit_ns, int arm) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1);
    fence_mbar_init();
    if (arm) {
        mbar_expect_tx(&bar, 16u);
    } else {
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&bar)) : "memory");
    }
    if (!mbar_wait_bounded(&bar, 0u, limit_ns)) atomicOr(status, PMGB_DEVERR_TMA_TIMEOUT);
}

cudaError_t pmgb_launch_bounded_wait_test(unsigned int* status, unsigned long long limit_ns, int arm,
                                          cudaStream_t st) {
    bounded_wait_test_kernel<<<1, 32, 0, st>>>(status, limit_ns, arm);
    return cudaGetLastError();
}

// Rotational energy grid values from the block results of its points: -T log(Σ e^{-U/T} / n)
// times the unit factor (+Inf where every orientation overlaps), src/grid.jl:338-351.
__global__ void rot_grid_out_kernel(const double* block_out, int n, double temperature, double log_n, double unit,
                                    float* out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const double L = block_out[4 * b];
    out[b] = isfinite(L) ? static_cast<float>(-temperature * (L - log_n) * unit) : __int_as_float(0x7f800000);
}

cudaError_t pmgb_launch_rot_grid_out(const double* block_out, int n, double temperature, double log_n, double unit,
                                     float* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    rot_grid_out_kernel<<<(n + 255) / 256, 256, 0, st>>>(block_out, n, temperature, log_n, unit, out);
    return cudaGetLastError();
}

cudaError_t pmgb_launch_fp32_peak(float* sink, int n_ctas, int iters, cudaStream_t st) {
    fp32_peak_kernel<<<n_ctas, 256, 0, st>>>(sink, iters);
    return cudaGetLastError();
}

// ============================================================================
// Fixed scratch for pmgb_widom_noalloc.
//
// Some callers cannot let the library call cudaMalloc / cudaFree during a run: cudaFree
// (and often cudaMalloc) synchronises the whole device, which stalls a host that keeps
// other work in flight on the same GPU, and processes whose device memory is already
// reserved by another allocator's pool (a Julia or Python framework's caching allocator)
// may have nothing left to hand out.  For them the per-CTA Boltzmann partials live in this
// file-scope array, reserved once when the library is loaded on a device.
// ============================================================================
namespace {
__device__ __align__(256) LsePartial g_noalloc_partials[PMGB_NOALLOC_MAX_CTAS];
}

// Device address of g_noalloc_partials on `device` (which must be current).  Host code must
// not use the symbol itself: on the host it names a stand-in, not device memory.  The
// lookup runs once per device and is cached in an atomic slot, so host threads with their
// own contexts may make their first calls concurrently (each may look the address up; all
// store the same value).  It allocates nothing.
cudaError_t pmgb_noalloc_scratch(int device, LsePartial** ptr) {
    static std::atomic<void*> cached[PMGB_NOALLOC_MAX_DEVICES] = {};
    if (device < 0 || device >= PMGB_NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
    void* p = cached[device].load(std::memory_order_acquire);
    if (!p) {
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess) return e;
        cached[device].store(p, std::memory_order_release);
    }
    *ptr = static_cast<LsePartial*>(p);
    return cudaSuccess;
}

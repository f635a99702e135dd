// pmgb_batch.cu -- persistent Widom screening of many frameworks in one launch.
//
// The batch is a list of systems (framework + guest) of uneven sizes.  Each system's
// insertions are cut into units of PMGB_THREADS (one statistics block at a time, as the
// single-system kernel does), and a grid of resident CTAs pulls units from one atomic
// counter in a host-chosen order (largest frameworks first by default), so that the
// tail of the launch is made of small units.  A CTA keeps its TMA ring between units and
// copies each unit's system descriptor into shared memory.  The adjoint variant reduces
// its Boltzmann-weighted r^-12 / r^-6 columns inside the unit (weights relative to the
// unit's own maximum of -U/T), so no per-insertion columns reach HBM; a per-system
// reduction combines units in a fixed order.
#include "pmgb_img.cuh"

namespace {

// (n_sites template, charged) of each compiled variant
constexpr int kVariantSites[6] = {1, 2, 3, 4, 6, 8};

// Each variant is its own function so that ptxas allocates its registers separately.
template <int NS, bool CHARGED, bool GRAD, bool RESID, bool COMP>
__device__ __noinline__ bool run_unit_fn(const SysDev& S, const UnitIO& io, int4* stage, uint64_t* bars,
                                         LsePartial* red, uint32_t (&fills)[PMGB_NSTAGE], unsigned int* status) {
    return run_unit<NS, CHARGED, GRAD, RESID, false, COMP>(S, io, stage, bars, red, fills, status);  // no forces
}

// one guest site: no centre-image variant (the site is the centre); the centre-image variant keeps
// the box-matrix residual whether or not refinement follows
template <int NS, bool CHARGED, bool GRAD, bool RESID>
__device__ __forceinline__ bool run_unit_c(bool comp, const SysDev& S, const UnitIO& io, int4* stage, uint64_t* bars,
                                           LsePartial* red, uint32_t (&fills)[PMGB_NSTAGE], unsigned int* status) {
    if constexpr (NS > 1)
        if (comp) return run_unit_fn<NS, CHARGED, GRAD, true, true>(S, io, stage, bars, red, fills, status);
    return run_unit_fn<NS, CHARGED, GRAD, RESID, false>(S, io, stage, bars, red, fills, status);
}

template <bool GRAD, bool RESID>
__device__ __forceinline__ bool run_variant_r(int variant, bool comp, const SysDev& S, const UnitIO& io, int4* stage,
                                              uint64_t* bars, LsePartial* red, uint32_t (&fills)[PMGB_NSTAGE],
                                              unsigned int* status) {
    switch (variant) {
        case 0: return run_unit_c<1, false, GRAD, RESID>(comp, S, io, stage, bars, red, fills, status);
        case 1: return run_unit_c<2, false, GRAD, RESID>(comp, S, io, stage, bars, red, fills, status);
        case 2: return run_unit_c<3, false, GRAD, RESID>(comp, S, io, stage, bars, red, fills, status);
        case 3: return run_unit_c<4, false, GRAD, RESID>(comp, S, io, stage, bars, red, fills, status);
        case 4: return run_unit_c<6, false, GRAD, RESID>(comp, S, io, stage, bars, red, fills, status);
        case 5: return run_unit_c<8, false, GRAD, RESID>(comp, S, io, stage, bars, red, fills, status);
        case 6: return run_unit_c<1, true, GRAD, RESID>(comp, S, io, stage, bars, red, fills, status);
        case 7: return run_unit_c<2, true, GRAD, RESID>(comp, S, io, stage, bars, red, fills, status);
        case 8: return run_unit_c<3, true, GRAD, RESID>(comp, S, io, stage, bars, red, fills, status);
        case 9: return run_unit_c<4, true, GRAD, RESID>(comp, S, io, stage, bars, red, fills, status);
        case 10: return run_unit_c<6, true, GRAD, RESID>(comp, S, io, stage, bars, red, fills, status);
        default: return run_unit_c<8, true, GRAD, RESID>(comp, S, io, stage, bars, red, fills, status);
    }
}

// the adjoint always keeps the box-matrix residual; comp: the centre-image variant (a guest with
// several sites where the system's geometry allows it, SysDev::com_axis)
template <bool GRAD>
__device__ __forceinline__ bool run_variant(int variant, bool no_resid, bool comp, const SysDev& S, const UnitIO& io,
                                            int4* stage, uint64_t* bars, LsePartial* red,
                                            uint32_t (&fills)[PMGB_NSTAGE], unsigned int* status) {
    if constexpr (!GRAD) {
        if (no_resid) return run_variant_r<false, false>(variant, comp, S, io, stage, bars, red, fills, status);
    }
    return run_variant_r<GRAD, true>(variant, comp, S, io, stage, bars, red, fills, status);
}

// image-list units (csrc/pmgb_img.cuh), one function per variant; COLS: with the adjoint's
// columns (the forward runs have none)
template <int NS, bool CHARGED, bool COLS>
__device__ __noinline__ void img_unit_fn(const SysDev& S, const UnitIO& io, unsigned char* smem) {
    img_unit<NS, CHARGED, false, COLS>(S, io, smem);
}

// the list takes the TMA ring's shared memory (idle here: every copy a unit issues is consumed
// inside that unit)
template <bool COLS>
__device__ __forceinline__ void run_img(const SysDev& S, const UnitIO& io, unsigned char* smem) {
    if (S.n_sites == 1) {
        if (S.charged) img_unit_fn<1, true, COLS>(S, io, smem);
        else img_unit_fn<1, false, COLS>(S, io, smem);
    } else {
        if (S.charged) img_unit_fn<3, true, COLS>(S, io, smem);
        else img_unit_fn<3, false, COLS>(S, io, smem);
    }
}

static_assert(sizeof(BatchSystem) % 4 == 0, "BatchSystem is copied to shared memory as 32-bit words");
static_assert(kImgSmemBytes <= size_t(PMGB_NSTAGE) * PMGB_TILE * sizeof(int4),
              "the image list fits in the TMA ring's shared memory");

template <bool GRAD>
__global__ void __launch_bounds__(PMGB_THREADS, 2) batch_kernel(const __grid_constant__ BatchArgs b) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    int4* stage = reinterpret_cast<int4*>(smem_raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + size_t(PMGB_NSTAGE) * PMGB_TILE * sizeof(int4));
    __shared__ LsePartial red[PMGB_THREADS / 32];
    __shared__ __align__(16) BatchSystem s_bs;
    __shared__ double s_m;
    __shared__ double s_wm[PMGB_THREADS / 32];
    __shared__ double s_w[GRAD ? PMGB_THREADS : 1];
    __shared__ int s_unit;
    const int tid = threadIdx.x;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    ring_init(bars);
    uint32_t fills[PMGB_NSTAGE] = {};
    const BatchRun run = *b.run;
    float* my_dsum = GRAD ? b.dsum + static_cast<size_t>(blockIdx.x) * b.max_cols * PMGB_THREADS : nullptr;
    for (;;) {
        if (tid == 0) s_unit = atomicAdd(b.counter, 1);
        __syncthreads();
        const int u = s_unit;
        if (u >= b.n_units) break;  // uniform: every thread read the same s_unit
        const BatchUnit unit = b.units[b.order[u]];
        {
            const int* src = reinterpret_cast<const int*>(b.systems + unit.system);
            int* dst = reinterpret_cast<int*>(&s_bs);
            for (int i = tid; i < static_cast<int>(sizeof(BatchSystem) / 4); i += PMGB_THREADS) dst[i] = src[i];
        }
        __syncthreads();
        const long long npb = s_bs.n_per_block;
        // a framework that fits the ring stays resident across the unit's chunks
        const bool fits = s_bs.sys.n_tiles <= PMGB_NSTAGE;
        for (int c = 0; c < unit.n_chunks; ++c) {
            const int chunk = unit.chunk0 + c;
            const int slot = s_bs.chunk_first + unit.block * s_bs.ctas_per_block + chunk;
            UnitIO io{};
            io.pose_mode = POSE_PHILOX;
            io.out_mode = OUT_WIDOM;
            const long long slot_in_block = static_cast<long long>(chunk) * PMGB_THREADS + tid;
            io.valid = slot_in_block < npb;
            long long within = slot_in_block;
            if (b.perm && io.valid)
                within = b.perm[s_bs.u_base + static_cast<long long>(unit.block) * npb + slot_in_block];
            double x = -inf;  // GRAD: this thread's -U/T
            if (s_bs.img) {
                // one order over the system's whole run: perm holds the system's insertion index
                io.item = io.valid ? within : 0;
                io.seed = run.seed + static_cast<unsigned long long>(unit.system) * 0x9E3779B97F4A7C15ull;
                io.u_out = b.u + 2 * s_bs.u_base;
                if (!GRAD) {
                    run_img<false>(s_bs.sys, io, smem_raw);
                    continue;
                }
                io.dsum = my_dsum;
                io.dsum_stride = PMGB_THREADS;
                io.col_item = tid;
                run_img<true>(s_bs.sys, io, smem_raw);
                if (io.valid) {  // the unit wrote this thread's energies; -U/T as run_unit forms it
                    const double uu = io.u_out[2 * io.item] + io.u_out[2 * io.item + 1];
                    if (isfinite(uu)) x = -uu * run.inv_temperature;
                }
            } else {
                io.item = static_cast<long long>(unit.block) * npb + within;
                io.cull = b.perm != nullptr;
                io.seed = run.seed + static_cast<unsigned long long>(unit.system) * 0x9E3779B97F4A7C15ull;
                io.inv_temperature = run.inv_temperature;
                io.dsum = my_dsum;
                io.dsum_stride = PMGB_THREADS;
                io.col_item = tid;
                io.partial = b.perm ? nullptr : b.partials + slot;
                io.u_out = b.u ? b.u + 2 * s_bs.u_base : nullptr;
                io.resident = fits && c > 0;
                io.x_out = &x;
                io.m_out = &s_m;
                const bool comp = s_bs.sys.com_axis >= -1 && s_bs.sys.n_sites > 1;
                if (!run_variant<GRAD>(s_bs.variant, b.no_resid != 0, comp, s_bs.sys, io, stage, bars, red, fills,
                                       b.status))
                    return;
            }
            if (GRAD) {
                if (b.perm) {
                    // this processing chunk's own max of -U/T (the partials come from u later)
                    double m = x;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
                    if ((tid & 31) == 0) s_wm[tid >> 5] = m;
                    __syncthreads();
                    if (tid == 0) {
                        double mm = s_wm[0];
                        for (int w = 1; w < PMGB_THREADS / 32; ++w) mm = fmax(mm, s_wm[w]);
                        s_m = mm;
                        b.unit_m[slot] = mm;
                    }
                }
                __syncthreads();  // s_m and every thread's columns are written
                const double M = s_m;
                s_w[tid] = (x == -inf || M == -inf) ? 0.0 : exp(x - M);
                __syncthreads();
                const int nc = s_bs.n_cols;
                double* out = b.unit_cols + s_bs.col_base + static_cast<long long>(slot - s_bs.chunk_first) * nc;
                const int warp = tid >> 5, lane = tid & 31;
                for (int cc = warp; cc < nc; cc += PMGB_THREADS / 32) {
                    const float* col = my_dsum + static_cast<size_t>(cc) * PMGB_THREADS;
                    double v = 0.0;
#pragma unroll
                    for (int i = lane; i < PMGB_THREADS; i += 32) {
                        const double w = s_w[i];
                        // w = 0 marks an empty slot or U = +Inf, whose column may be garbage or Inf
                        if (w > 0.0) v = fma(w, static_cast<double>(col[i]), v);
                    }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                    if (lane == 0) out[cc] = v;
                }
            }
            __syncthreads();  // red, s_m, s_w and the columns are free for the next chunk
        }
        __syncthreads();  // s_bs, s_w and the ring are free for the next unit
    }
}

// One CTA per system: block results (as reduce_blocks_kernel) and, with the adjoint, the
// combined columns relative to m = max over the system's chunks of max -U/T.
__global__ void batch_reduce_kernel(const BatchSystem* __restrict__ systems, int n_blocks,
                                    const LsePartial* __restrict__ partials, const double* __restrict__ unit_cols,
                                    const double* __restrict__ unit_m, bool grad, double* __restrict__ block_out,
                                    double* __restrict__ out_cols) {
    const int s = blockIdx.x;
    const BatchSystem& bs = systems[s];
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    const unsigned full = 0xffffffffu;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nw = blockDim.x >> 5;
    const int cpb = bs.ctas_per_block;
    for (int blk = warp; blk < n_blocks; blk += nw) {
        const LsePartial* p = partials + bs.chunk_first + static_cast<size_t>(blk) * cpb;
        double m = -inf;
        for (int c = lane; c < cpb; c += 32) m = fmax(m, p[c].m);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(full, m, o));
        double sum = 0.0, tv = 0.0, te = 0.0;
        long long n = 0;
        for (int c = lane; c < cpb; c += 32) {
            const LsePartial q = p[c];
            const double f = (m == -inf || q.m == -inf) ? 0.0 : exp(q.m - m);
            sum += q.s * f;
            tv += q.tv * f;
            te += q.te * f;
            n += q.n_inf;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sum += __shfl_xor_sync(full, sum, o);
            tv += __shfl_xor_sync(full, tv, o);
            te += __shfl_xor_sync(full, te, o);
            n += __shfl_xor_sync(full, n, o);
        }
        if (lane == 0) {
            double* o = block_out + (static_cast<size_t>(s) * n_blocks + blk) * 4;
            o[0] = (sum > 0.0) ? m + log(sum) : -inf;
            o[1] = tv / sum;
            o[2] = te / sum;
            o[3] = static_cast<double>(n);
        }
    }
    if (!grad) return;
    __shared__ double s_max;
    const int n_units = n_blocks * cpb;
    const LsePartial* p = partials + bs.chunk_first;
    if (warp == 0) {
        double m = -inf;
        for (int c = lane; c < n_units; c += 32) m = fmax(m, p[c].m);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(full, m, o));
        if (lane == 0) s_max = m;
    }
    __syncthreads();
    const double M = s_max;
    const int nc = bs.n_cols;
    double* out = out_cols + bs.out_base;
    // entry e: 0 -> M, 1 -> sum w, 2 -> sum w U_es, 3 + c -> sum w col_c; units in a fixed order
    for (int e = threadIdx.x; e < 3 + nc; e += blockDim.x) {
        if (e == 0) {
            out[0] = M;
            continue;
        }
        double v = 0.0;
        for (int k = 0; k < n_units; ++k) {
            // columns were weighted relative to their processing chunk's max (unit_m with a spatial
            // order, else the same chunk's partial)
            const double mk = (e >= 3 && unit_m) ? unit_m[bs.chunk_first + k] : p[k].m;
            const double f = (M == -inf || mk == -inf) ? 0.0 : exp(mk - M);
            if (f == 0.0) continue;
            const double x = (e == 1) ? p[k].s : (e == 2) ? p[k].te : unit_cols[bs.col_base + static_cast<size_t>(k) * nc + (e - 3)];
            v = fma(f, x, v);
        }
        out[e] = v;
    }
}

// ---- spatial order of a batch ------------------------------------------------------------
constexpr int kBatchOrderBits = 4;                           // 16 cells per axis
constexpr int kBatchOrderCells = 1 << (3 * kBatchOrderBits);  // 4096

// Hilbert-curve cell of insertion idx (the top 4 bits of each centre-of-mass coordinate)
__device__ __forceinline__ int batch_cell(unsigned long long seed, unsigned long long idx) {
    const uint2 key = make_uint2(static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    const uint4 a = philox4x32_10(make_uint4(static_cast<uint32_t>(idx), static_cast<uint32_t>(idx >> 32), 0u, 0u), key);
    return hilbert_cell(a.x >> (32 - kBatchOrderBits), a.y >> (32 - kBatchOrderBits), a.z >> (32 - kBatchOrderBits),
                        kBatchOrderBits);
}

struct ChunkRef {
    int sys, blk;
    long long within, npb;
    bool valid;
};

__device__ __forceinline__ ChunkRef chunk_ref(const BatchSystem* systems, const int* chunk_sys, int c, int tid) {
    ChunkRef r;
    r.sys = chunk_sys[c];
    const BatchSystem& bs = systems[r.sys];
    const int local = c - bs.chunk_first;
    r.blk = local / bs.ctas_per_block;
    r.within = static_cast<long long>(local % bs.ctas_per_block) * PMGB_THREADS + tid;
    r.npb = bs.n_per_block;
    r.valid = r.within < r.npb;
    return r;
}

__global__ void batch_order_count_kernel(const BatchSystem* systems, const int* chunk_sys, int n_blocks,
                                         const BatchRun* run, int* counts) {
    const ChunkRef r = chunk_ref(systems, chunk_sys, blockIdx.x, threadIdx.x);
    if (!r.valid || systems[r.sys].img) return;
    const unsigned long long seed = run->seed + static_cast<unsigned long long>(r.sys) * 0x9E3779B97F4A7C15ull;
    const int cell = batch_cell(seed, static_cast<unsigned long long>(r.blk * r.npb + r.within));
    atomicAdd(&counts[(static_cast<size_t>(r.sys) * n_blocks + r.blk) * kBatchOrderCells + cell], 1);
}

// exclusive scan of one (system, block)'s 4096 cell counts
__global__ void __launch_bounds__(1024) batch_order_scan_kernel(int* counts) {
    __shared__ int part[1024];
    int* c = counts + static_cast<size_t>(blockIdx.x) * kBatchOrderCells;
    constexpr int per = kBatchOrderCells / 1024;
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

__global__ void batch_order_scatter_kernel(const BatchSystem* systems, const int* chunk_sys, int n_blocks,
                                           const BatchRun* run, int* offsets, int* perm) {
    const ChunkRef r = chunk_ref(systems, chunk_sys, blockIdx.x, threadIdx.x);
    if (!r.valid || systems[r.sys].img) return;
    const unsigned long long seed = run->seed + static_cast<unsigned long long>(r.sys) * 0x9E3779B97F4A7C15ull;
    const int cell = batch_cell(seed, static_cast<unsigned long long>(r.blk * r.npb + r.within));
    const int pos = atomicAdd(&offsets[(static_cast<size_t>(r.sys) * n_blocks + r.blk) * kBatchOrderCells + cell], 1);
    perm[systems[r.sys].u_base + r.blk * r.npb + pos] = static_cast<int>(r.within);
}

// ---- one order over each image-list system's run (the single-system order, csrc/pmgb_img.cu) ----
__global__ void batch_run_count_kernel(const BatchSystem* systems, const int* chunk_sys, const BatchRun* run,
                                       int* cells) {
    const ChunkRef r = chunk_ref(systems, chunk_sys, blockIdx.x, threadIdx.x);
    if (!r.valid) return;
    const BatchSystem& bs = systems[r.sys];
    if (!bs.img) return;
    const unsigned long long seed = run->seed + static_cast<unsigned long long>(r.sys) * 0x9E3779B97F4A7C15ull;
    atomicAdd(&cells[bs.cell_base + run_cell(seed, static_cast<unsigned long long>(r.blk * r.npb + r.within),
                                             bs.order_bits)], 1);
}

// exclusive scan of one image-list system's cells (CTA s: system s)
__global__ void __launch_bounds__(1024) batch_run_scan_kernel(const BatchSystem* systems, int* cells) {
    const BatchSystem& bs = systems[blockIdx.x];
    if (!bs.img) return;  // uniform over the CTA
    scan_cells(cells + bs.cell_base, 1 << (3 * bs.order_bits));
}

__global__ void batch_run_scatter_kernel(const BatchSystem* systems, const int* chunk_sys, const BatchRun* run,
                                         int* cells, int* perm) {
    const ChunkRef r = chunk_ref(systems, chunk_sys, blockIdx.x, threadIdx.x);
    if (!r.valid) return;
    const BatchSystem& bs = systems[r.sys];
    if (!bs.img) return;
    const unsigned long long seed = run->seed + static_cast<unsigned long long>(r.sys) * 0x9E3779B97F4A7C15ull;
    const long long idx = r.blk * r.npb + r.within;
    const int pos = atomicAdd(&cells[bs.cell_base + run_cell(seed, static_cast<unsigned long long>(idx), bs.order_bits)], 1);
    perm[bs.u_base + pos] = static_cast<int>(idx);
}

// each cell's insertions by index (CTA s: system s; cells[c] is the end of cell c after the scatter)
__global__ void batch_run_sort_kernel(const BatchSystem* systems, const int* cells, int* perm) {
    const BatchSystem& bs = systems[blockIdx.x];
    if (!bs.img) return;
    const int n_cells = 1 << (3 * bs.order_bits);
    const int* end = cells + bs.cell_base;
    int* p = perm + bs.u_base;
    for (int c = threadIdx.x; c < n_cells; c += blockDim.x) {
        const int lo = c == 0 ? 0 : end[c - 1], hi = end[c];
        for (int i = lo + 1; i < hi; ++i) {
            const int v = p[i];
            int j = i - 1;
            while (j >= lo && p[j] > v) {
                p[j + 1] = p[j];
                --j;
            }
            p[j + 1] = v;
        }
    }
}

// per-chunk log-sum-exp partials in insertion order (what the kernel forms without a spatial order)
__global__ void __launch_bounds__(PMGB_THREADS) batch_lse_kernel(const BatchSystem* systems, const int* chunk_sys,
                                                                const BatchRun* run, const double* __restrict__ u,
                                                                LsePartial* __restrict__ partials) {
    __shared__ LsePartial red[PMGB_THREADS / 32];
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    const ChunkRef r = chunk_ref(systems, chunk_sys, blockIdx.x, threadIdx.x);
    double x = -inf, ev = 0.0, ee = 0.0;
    long long ninf = 0;
    if (r.valid) {
        const long long ui = systems[r.sys].u_base + r.blk * r.npb + r.within;
        const double uv = u[2 * ui], ues = u[2 * ui + 1];
        const double uu = uv + ues;
        if (isfinite(uu)) {
            x = -uu * run->inv_temperature;
            ev = uv;
            ee = ues;
        } else {
            ninf = 1;
        }
    }
    lse_cta(x, ev, ee, ninf, red, partials + blockIdx.x, nullptr);
}

}  // namespace

size_t pmgb_batch_order_cells() { return kBatchOrderCells; }

cudaError_t pmgb_launch_batch_order(const BatchSystem* systems, const int* chunk_sys, int n_chunks, int n_systems,
                                    int n_blocks, const BatchRun* run, int* counts, int* perm, cudaStream_t st) {
    const size_t n_counts = static_cast<size_t>(n_systems) * n_blocks * kBatchOrderCells;
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * n_counts, st);
    if (e != cudaSuccess) return e;
    batch_order_count_kernel<<<n_chunks, PMGB_THREADS, 0, st>>>(systems, chunk_sys, n_blocks, run, counts);
    batch_order_scan_kernel<<<n_systems * n_blocks, 1024, 0, st>>>(counts);
    batch_order_scatter_kernel<<<n_chunks, PMGB_THREADS, 0, st>>>(systems, chunk_sys, n_blocks, run, counts, perm);
    return cudaGetLastError();
}

cudaError_t pmgb_launch_batch_run_order(const BatchSystem* systems, const int* chunk_sys, int n_chunks, int n_systems,
                                        const BatchRun* run, int* cells, long long n_cells, int* perm, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(cells, 0, sizeof(int) * static_cast<size_t>(n_cells), st);
    if (e != cudaSuccess) return e;
    batch_run_count_kernel<<<n_chunks, PMGB_THREADS, 0, st>>>(systems, chunk_sys, run, cells);
    batch_run_scan_kernel<<<n_systems, 1024, 0, st>>>(systems, cells);
    batch_run_scatter_kernel<<<n_chunks, PMGB_THREADS, 0, st>>>(systems, chunk_sys, run, cells, perm);
    batch_run_sort_kernel<<<n_systems, 256, 0, st>>>(systems, cells, perm);
    return cudaGetLastError();
}

cudaError_t pmgb_launch_batch_lse(const BatchSystem* systems, const int* chunk_sys, int n_chunks, const BatchRun* run,
                                  const double* u, LsePartial* partials, cudaStream_t st) {
    batch_lse_kernel<<<n_chunks, PMGB_THREADS, 0, st>>>(systems, chunk_sys, run, u, partials);
    return cudaGetLastError();
}

int pmgb_batch_variant(int n_sites, bool charged) {
    for (int i = 0; i < 6; ++i)
        if (n_sites <= kVariantSites[i]) return i + (charged ? 6 : 0);
    return -1;
}

cudaError_t pmgb_batch_prepare(bool grad) {
    const int smem = static_cast<int>(pmgb_pairs_smem_bytes());
    return grad ? cudaFuncSetAttribute(batch_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)
                : cudaFuncSetAttribute(batch_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

cudaError_t pmgb_launch_batch(const BatchArgs& b, bool grad, int n_ctas, cudaStream_t st) {
    const size_t smem = pmgb_pairs_smem_bytes();
    if (grad) batch_kernel<true><<<n_ctas, PMGB_THREADS, smem, st>>>(b);
    else batch_kernel<false><<<n_ctas, PMGB_THREADS, smem, st>>>(b);
    return cudaGetLastError();
}

cudaError_t pmgb_launch_batch_reduce(const BatchSystem* systems, int n_systems, int n_blocks,
                                     const LsePartial* partials, const double* unit_cols, const double* unit_m,
                                     bool grad, double* block_out, double* out_cols, cudaStream_t st) {
    if (n_systems <= 0) return cudaSuccess;
    batch_reduce_kernel<<<n_systems, 128, 0, st>>>(systems, n_blocks, partials, unit_cols, unit_m, grad, block_out,
                                                   out_cols);
    return cudaGetLastError();
}

// pmgb_img.cu -- the image-list form of the spatially ordered Widom pass (sm_103a).
//
// The insertions of a run are sorted once over the whole run (all statistics blocks) by the cell
// of their centre of mass along a Hilbert curve, so the 256 insertions of a CTA (and the 32 lanes
// of each of its warps) sit close together.  Each CTA takes the centre c of its guest sites'
// bounding box and the largest distance rho of a site from c, and gathers from the framework
// records (read from global memory, L2-resident; each thread takes one record per pass) every
// periodic image within R = r_cut + rho of c, as a double-float Cartesian offset from c, into a
// shared-memory list.  Every lane of every warp evaluates its guest sites against that list: a
// distance is three subtractions and a dot product, with no integer wrap or conversion per site,
// and records beyond R of every lane are never looked at.
//
// Why the sums are the reference's minimum-image sums (src/vdw_energetics.jl:25-47,
// src/electrostatics.jl:377-386): every perpendicular width of the supercell exceeds twice the
// larger cutoff (the caller checks), so a site has at most one image of a record within the
// cutoff, and that image is its minimum image.  A site lies within rho of c, so such an image lies
// within R of c and is in the list; the other images in the list lie beyond the cutoff of that
// site and contribute exact zeros.  The list is built from the records in their stored order (per
// species segment), so it and every sum over it are deterministic; the sort orders the insertions
// of a cell by index, so the warps' compositions are deterministic too.
//
// Precision: the list holds each offset's FP32 value and its FP32 residual (value + residual is
// the minimum-image offset to ~1e-13 A); distances take the values, and pairs closer than 4 A add
// the residuals' first-order term, so the energies keep the per-site pass's FP32 error bound
// against FP64, with or without the FP64 tail refinement.
#include "pmgb_img.cuh"

namespace {

// ---- spatial order over a whole run (run_cell: csrc/pmgb_img.cuh) ---------------------------
__global__ void run_order_count_kernel(unsigned long long seed, long long n, int bits, int* counts) {
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    atomicAdd(&counts[run_cell(seed, static_cast<unsigned long long>(i), bits)], 1);
}

// exclusive scan of the run's cell counts (one CTA of 1024 threads)
__global__ void __launch_bounds__(1024) run_order_scan_kernel(int* counts, int n_cells) { scan_cells(counts, n_cells); }

__global__ void run_order_scatter_kernel(unsigned long long seed, long long n, int bits, int* offsets, int* perm) {
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int pos = atomicAdd(&offsets[run_cell(seed, static_cast<unsigned long long>(i), bits)], 1);
    perm[pos] = static_cast<int>(i);
}

// The scatter leaves each cell's insertions in atomic order; sort every cell's slice by insertion
// index so that the processing order, and with it each warp's list, is the same on every run.
// offsets[c] is the end of cell c after the scatter.
__global__ void run_order_sort_kernel(const int* offsets, int n_cells, int* perm) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cells) return;
    const int lo = c == 0 ? 0 : offsets[c - 1], hi = offsets[c];
    for (int i = lo + 1; i < hi; ++i) {
        const int v = perm[i];
        int j = i - 1;
        while (j >= lo && perm[j] > v) {
            perm[j + 1] = perm[j];
            --j;
        }
        perm[j + 1] = v;
    }
}

template <int NS, bool CHARGED, bool STATS, bool COLS>
__global__ void __launch_bounds__(PMGB_THREADS, 2) pairs_img_kernel(const __grid_constant__ LaunchArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];

    UnitIO io{};
    io.pose_mode = POSE_PHILOX;
    io.out_mode = OUT_WIDOM;
    // CTA (block b, chunk c) takes slots b n_per_block + c 256 + [0, 256) of the run's order, as
    // the batch kernel's units do, so that a system's warps hold the same insertions in both
    const int b = blockIdx.x / a.ctas_per_block;
    const long long slot = static_cast<long long>(blockIdx.x % a.ctas_per_block) * PMGB_THREADS + threadIdx.x;
    io.valid = slot < a.n_per_block;
    io.item = io.valid ? a.perm[static_cast<long long>(b) * a.n_per_block + slot] : 0;
    io.seed = a.seed;
    io.u_out = a.u_out;
    io.stats = a.stats;
    if (COLS) {
        io.dsum = a.dsum;
        io.dsum_stride = a.dsum_stride;
        io.col_item = io.item;
    }
    img_unit<NS, CHARGED, STATS, COLS>(a.sys, io, smem_raw);
}

template <int NS, bool CH, bool STATS, bool COLS = false>
cudaError_t launch_img(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    const size_t smem = pmgb_img_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(pairs_img_kernel<NS, CH, STATS, COLS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    pairs_img_kernel<NS, CH, STATS, COLS><<<n_ctas, PMGB_THREADS, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace

size_t pmgb_img_smem_bytes() { return kImgSmemBytes; }

extern "C" int pmgb_hilbert_cell(uint32_t x, uint32_t y, uint32_t z, int32_t bits) {
    if (bits < 1 || bits > 10 || (x >> bits) || (y >> bits) || (z >> bits)) return -1;
    return hilbert_cell(x, y, z, bits);
}

bool pmgb_img_supported(int n_sites) { return n_sites == 1 || n_sites == 3; }

// Cells per axis 2^bits: the fewest bits (3 to 6) that leave at most 32 insertions per cell
// on average (a cell of a 1e6-insertion run in a 28,700 A^3 cell is ~0.9 A across; the order within
// a cell is by index)
int pmgb_run_order_bits(long long n) {
    int bits = 3;
    while (bits < 6 && (n >> (3 * bits)) > 32) ++bits;
    return bits;
}

cudaError_t pmgb_launch_run_order(unsigned long long seed, long long n, int* counts, int* perm, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int bits = pmgb_run_order_bits(n);
    const int n_cells = 1 << (3 * bits);
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * static_cast<size_t>(n_cells), st);
    if (e != cudaSuccess) return e;
    const unsigned grid = static_cast<unsigned>((n + 255) / 256);
    run_order_count_kernel<<<grid, 256, 0, st>>>(seed, n, bits, counts);
    run_order_scan_kernel<<<1, 1024, 0, st>>>(counts, n_cells);
    run_order_scatter_kernel<<<grid, 256, 0, st>>>(seed, n, bits, counts, perm);
    run_order_sort_kernel<<<(n_cells + 255) / 256, 256, 0, st>>>(counts, n_cells, perm);
    return cudaGetLastError();
}

cudaError_t pmgb_launch_pairs_img(const LaunchArgs& a, int n_ctas, cudaStream_t st) {
    if (n_ctas <= 0) return cudaSuccess;
    if (!a.perm || !a.u_out || a.pose_mode != POSE_PHILOX) return cudaErrorInvalidValue;
    const bool stats = a.stats != nullptr;
    if (a.dsum) {  // the adjoint's columns (no work counting)
        if (stats) return cudaErrorInvalidValue;
        if (a.sys.n_sites == 1)
            return a.sys.charged ? launch_img<1, true, false, true>(a, n_ctas, st) : launch_img<1, false, false, true>(a, n_ctas, st);
        if (a.sys.n_sites == 3)
            return a.sys.charged ? launch_img<3, true, false, true>(a, n_ctas, st) : launch_img<3, false, false, true>(a, n_ctas, st);
        return cudaErrorNotSupported;
    }
    if (a.sys.n_sites == 1) {
        if (a.sys.charged) return stats ? launch_img<1, true, true>(a, n_ctas, st) : launch_img<1, true, false>(a, n_ctas, st);
        return stats ? launch_img<1, false, true>(a, n_ctas, st) : launch_img<1, false, false>(a, n_ctas, st);
    }
    if (a.sys.n_sites == 3) {
        if (a.sys.charged) return stats ? launch_img<3, true, true>(a, n_ctas, st) : launch_img<3, true, false>(a, n_ctas, st);
        return stats ? launch_img<3, false, true>(a, n_ctas, st) : launch_img<3, false, false>(a, n_ctas, st);
    }
    return cudaErrorNotSupported;
}

// pmgb_internal.h -- device data layout shared by the kernels and the C-ABI layer.
//
// Layout in HBM (all owned by a pmgb_system):
//   rec[n_rec]      int4 (x, y, z, q) of every framework site of the replicated crystal:
//                   fractional coordinates as 32-bit fixed point (x * 2^32 mod 2^32) and
//                   the charge as FP32 bits, sorted by LJ species into contiguous segments.
//   seg[n_seg]      [lo, hi) record range of each species segment.
//   segpar[n_seg * PMGB_MAX_SITES]  per (segment, guest site): sigma^2, 4*epsilon,
//                   overlap radius^2 (0.1, or -1 when the pair has no LJ term), 4 eps sigma^12
//                   and -4 eps sigma^6.
//   krow[n_krow]    k-vectors grouped in half-rows of constant (ka, kb) running outward in
//                   kc from the kc nearest 0.
//   skw[n_k]        wt_k * S(k) in half-row traversal order, FP32 (re, im); S(k) is
//                   accumulated on the device in FP64.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <vector>

#define PMGB_MAX_SITES 8      // guest sites (merged LJ atoms + point charges)
#define PMGB_MAX_SEG 64       // framework species segments
#define PMGB_TILE 2048        // framework records per shared-memory stage (32 KB)
#define PMGB_NSTAGE 3         // stages in the TMA ring
#define PMGB_THREADS 256      // insertions per CTA (one per thread)
#define PMGB_CHUNK 64         // framework records per compensated fold
#define PMGB_SUBCHUNK 16      // framework records per bounding box (chunks are cut into these)
#define PMGB_ES_COEF 8        // coefficients per interval of the FP64 erfc(alpha r)/r table
#define PMGB_ES_SUB 32        // intervals per octave of r^2 in that table
#define PMGB_ES_E_LO (-7)     // the table starts at r^2 = 2^-7 A^2 (closer pairs: direct formula)

// status word bits written by kernels (never a trap)
#define PMGB_DEVERR_TMA_TIMEOUT 0x1u
#define PMGB_DEVERR_BAD_ARGS 0x2u

struct SegDesc {
    int lo, hi;        // record range [lo, hi)
    int species;       // species id in the caller's force-field table (-1: charge-only sites)
    int has_lj;
};

// Fixed-point bounding box of one sub-chunk of PMGB_SUBCHUNK framework records: centre and
// half-extent per axis, as 32-bit fractions of the supercell.
struct ChunkBox {
    uint32_t cx, cy, cz, pad0;
    uint32_t ex, ey, ez, pad1;
};

struct SitePar {
    float sig2, eps4, r2ovl;
    float lj12, lj6;   // 4 eps sigma^12 and -4 eps sigma^6 (so that U = r^-6 (lj12 r^-6 + lj6))
    float pad0, pad1, pad2;
};

struct KRow {
    // k = (ks0 ka, ks1 kb, ks2 (kc0 + dir * m)) for m = 0 .. n-1, ks = SysDev::ks
    int ka, kb, kc0, n;
    int off;              // index of the first k-vector of the row in skw (traversal order)
    int dir;              // +1 or -1
    int pad1, pad2;
};

// Everything a kernel needs to know about one (framework, guest) system.
struct SysDev {
    const int4* rec;
    int n_rec, n_tiles;
    // sub-chunk boxes in the kernels' traversal order (tiles, segments, chunks, sub-chunks)
    // and the perpendicular widths of the supercell per fixed-point step; cw_inv_lam = 1 / an
    // upper bound of the largest eigenvalue of the Gram matrix of the unit face normals
    const ChunkBox* cbox;
    float cw[3], cw_inv_lam;
    int n_seg;
    const SegDesc* seg;
    const SitePar* segpar;
    // upper-triangular f_to_c scaled by 2^-32 (Cartesian = H' * fixed-point displacement)
    // and c_to_f (unscaled), FP32
    float h00, h01, h02, h11, h12, h22;
    float p00, p01, p02, p11, p12, p22;   // FP32 residual of the scaled f_to_c (h + p = FP64 value)
    float g00, g01, g02, g11, g12, g22;
    float rc2;                     // LJ cutoff radius^2 (ljff.r²_cutoff)
    float rc2e;                    // Ewald real-space cutoff radius^2
    float alpha;                   // Ewald convergence parameter (1/A)
    double coul;                   // 1 / (4 pi eps0) in K A / e^2
    int charged;                   // guest-host electrostatics on
    // guest: site offsets from the centre of mass (Cartesian, A), charges
    int n_sites;
    float body[PMGB_MAX_SITES][3];
    float q[PMGB_MAX_SITES];
    float com_reach;               // largest distance of a guest site from the pose centre (A)
    // centre-image geometry (set with the cutoffs): com_axis -1 = the pose centre's minimum image
    // serves every guest site, -2 = per-site images only; com_reach2 = (larger cutoff + com_reach)^2
    int com_axis;
    float com_reach2;
    // Ewald reciprocal space
    int n_krow, n_k;
    const KRow* krow;
    const float2* skw;
    // k-vector strides: when the framework is a replicated cell, S(k) vanishes unless every
    // k_d is a multiple of the replication factor n_d, and only those k-vectors are kept;
    // rows then hold k / ks and the kernels evaluate them at the coordinates ks_d u_d
    int ks[3];
    // 1: three sites, site 0 at the centre of mass and sites 1 and 2 its mirror images through it
    // with equal charges (CO2): their fixed-point offsets from site 0 are exact negatives, so the
    // reciprocal-space sum needs the phase factor of site 1 only
    int k_mirror;
    // FP64 copies: guest poses are composed in FP64, and the Boltzmann-tail refinement
    // re-evaluates selected insertions entirely in FP64
    double f2c64[6];                        // f_to_c, upper triangular (00 01 02 11 12 22)
    double g64[6];                          // c_to_f, upper triangular
    double body64[PMGB_MAX_SITES][3];       // guest site offsets (Cartesian, A)
    double q64[PMGB_MAX_SITES];             // guest site charges
    double rc2_64, rc2e_64, alpha64;
    const double* rec_q;                    // [n_rec] framework charge of each record
    const double* rec_xf;                   // [3 n_rec] exact fractional coordinates of each record
    const double2* segpar64;                // [n_seg * PMGB_MAX_SITES] (sigma^2, 4 epsilon); 4 eps = 0: no LJ
    const double* sk64;                     // [2 n_k] S(k) (re, im) in half-row order
    const double* wt64;                     // [n_k] k-vector weights in half-row order
    const int* kabc;                        // [3 n_k] k-vectors in half-row order
    // erfc(alpha r) / r as a function of s = r^2 for the FP64 refinement: per interval
    // [2^e (1 + m/32), 2^e (1 + (m+1)/32)), e >= es_e_lo, m < 32, a degree-7 polynomial in
    // t = 64 x - (65 + 2 m) (x = s 2^-e), PMGB_ES_COEF coefficients from t^0 up
    const double* es_tab;
    int es_e_lo, es_n_oct;
    // double-float copies (value = hi + lo, two FP32 numbers, ~48 significant bits) for the
    // refinement's near-pair terms, which run on the FP32 pipes
    const float4* rec_rq;                   // [n_rec] x, y, z beyond the 32-bit fixed point (units of 2^-32), q hi
    const float* rec_qlo;                   // [n_rec] q lo
    const float4* segpar_df;                // [n_seg * PMGB_MAX_SITES] sigma^2 (hi, lo), 4 eps (hi, lo)
    const float2* es_tab_df;                // es_tab as (hi, lo)
    const float4* tk_df;                    // [n_k] wt_k S(k) (re hi, re lo, im hi, im lo), half-row order
    float2 h_df[6];                         // f2c64 * 2^-32: Cartesian per fixed-point unit
    float2 rc2_df, rc2e_df;
    // optional accessibility gate (src/henry.jl:225): blocked insertions get U = +Inf
    const uint8_t* acc;                     // [acc_n0 * acc_n1 * acc_n2], i fastest; 0 = inaccessible
    int acc_n[3];                           // grid points per axis of the unit-cell grid
    int acc_rep[3];                         // replication factors of the supercell
};

enum PoseMode : int {
    POSE_PHILOX = 0,   // Widom: pose of insertion i from Philox4x32-10(seed, i)
    POSE_SITES = 1,    // explicit site coordinates (n x n_sites x 3, FP64)
    POSE_GRID = 2,     // energy-grid points (single-site probe)
};

enum OutMode : int {
    OUT_WIDOM = 0,     // per-CTA Boltzmann partial sums (+ optional per-insertion U)
    OUT_ENERGY = 1,    // per-configuration (U_vdw, U_es_sr, U_es_lr)
    OUT_GRID = 2,      // per-point energy (float) * unit factor
};

// Per-CTA partial of the Boltzmann accumulation, log-sum-exp form.
struct LsePartial {
    double m;      // max of -U/T
    double s;      // sum exp(-U/T - m)
    double tv;     // sum U_vdw exp(-U/T - m)
    double te;     // sum U_es exp(-U/T - m)
    long long n_inf;  // insertions with U = +Inf (overlap)
    long long pad;
};

struct LaunchArgs {
    SysDev sys;
    int pose_mode, out_mode;
    // Widom (POSE_PHILOX)
    unsigned long long seed;
    long long n_per_block;       // insertions per statistics block
    int n_blocks;                // statistics blocks
    int ctas_per_block;          // CTAs covering one statistics block
    double inv_temperature;
    LsePartial* partials;        // [n_blocks * ctas_per_block]; NULL with perm (reduced from u_out)
    double* u_out;               // optional: [n_total * 2] (U_vdw, U_es); required with perm
    const int* perm;             // optional: processing order within each block (spatially sorted),
                                 //   slot s of block b evaluates insertion b * n_per_block + perm[..]
    // explicit sites (POSE_SITES)
    const uint32_t* site_fix;    // [n_conf * n_sites * 3] fixed-point fractional coordinates
    long long n_conf;
    const int* n_conf_dev;       // optional: n_conf read from device memory (latency path)
    double* e_out;               // [n_conf * 3] (vdw, sr, lr)
    // grid (POSE_GRID)
    int n_pts[3];
    const uint32_t* grid_x;      // fixed-point fractional coordinate of each grid plane, per
    const uint32_t* grid_y;      //   axis, already divided by the replication factor
    const uint32_t* grid_z;
    float unit_factor;
    float* grid_out;
    int grid_bricks;             // warps take 4 x 4 x 2 bricks of points (spatially compact)
    // rotational energy grid (POSE_PHILOX): block b's insertions sit at grid point point_base + b
    // (planes grid_x/y/z, n_pts) with rotations from Philox counters item_base + item; warps skip
    // out-of-cutoff terms (their lanes share the centre) without a processing order
    int rot_grid;
    long long point_base, item_base;
    // forward Widom whose Boltzmann tail is refined in FP64: distances from the FP32 box matrix
    // alone (no residual), ~13% less work; the refinement re-evaluates the insertions that matter
    int no_resid;
    // adjoint (GRAD kernels)
    float* dsum;                 // [(seg * NS + site) * 2 + {0: sum r^-12, 1: sum r^-6}][item], within cutoff
    long long dsum_stride;       // items per column
    float* grad_u;               // optional: [item * 3] dU/dx of the centre of mass (K/A)
    // energy grid with error scale (pmgb_launch_grid_bound)
    float* bound_out;            // [item] FP32 rounding-error estimate (K), +Inf where a pair sits at a threshold
    float bound_rho, bound_stat; // factors of the estimate (run_unit, BOUND)
    // work counts (pmgb_launch_pairs_stats)
    unsigned long long* stats;   // [3] distances evaluated, LJ and real-space terms inside their cutoffs
    // status
    unsigned int* status;
};

cudaError_t pmgb_launch_max_neg_u(const double* u, long long n, double inv_t, double* out, cudaStream_t st);
// Few explicit configurations (POSE_SITES, OUT_ENERGY), one CTA each with the framework split
// over its threads: the latency path of Monte Carlo moves.
cudaError_t pmgb_launch_energies_latency(const LaunchArgs& a, int n_ctas, cudaStream_t st);
// Spatial processing order of a Widom run: per block, a counting sort of the insertions by the
// Z-order cell (32^3 cells) of their centre of mass.  counts: [n_blocks * 32768] scratch;
// perm: [n_blocks * n_per_block] within-block insertion indices in processing order.
cudaError_t pmgb_launch_widom_order(unsigned long long seed, long long n_per_block, int n_blocks, int* counts,
                                    int* perm, cudaStream_t st);
size_t pmgb_widom_order_cells();
// Image-list Widom pass (csrc/pmgb_img.cu): one spatial order over a whole run (counts: scratch of
// 2^(3 bits) cells, bits = pmgb_run_order_bits(n); perm: [n] insertion indices in processing
// order, each cell's insertions by index), and the pass itself (a.perm, a.u_out required; one
// CTA per PMGB_THREADS slots of perm; a.stats set: the work-counting variant).
int pmgb_run_order_bits(long long n);
cudaError_t pmgb_launch_run_order(unsigned long long seed, long long n, int* counts, int* perm, cudaStream_t st);
bool pmgb_img_supported(int n_sites);
size_t pmgb_img_smem_bytes();
cudaError_t pmgb_launch_pairs_img(const LaunchArgs& a, int n_ctas, cudaStream_t st);
// Per-CTA log-sum-exp partials of a Widom run from its per-insertion energies, in insertion
// order (the partials the pair kernel forms itself when it runs without a permutation).
cudaError_t pmgb_launch_lse_from_u(const double* u, long long n_per_block, int n_blocks, int ctas_per_block,
                                   double inv_temperature, LsePartial* partials, cudaStream_t st);
// CTAs covering a grid of n_pts points taken in 4 x 4 x 2 bricks per warp
int pmgb_grid_brick_ctas(const int n_pts[3]);
// Weighted sums of per-item adjoint columns: out[c] = sum_i w_i col_c[i], w_i = exp(-U_i/T - M)
cudaError_t pmgb_launch_weighted_columns(const double* u, int u_stride, long long n, double inv_t,
                                         const double* log_scale, int n_log, const float* cols,
                                         int n_cols, long long col_stride, double* partials, int n_chunks,
                                         double* out, cudaStream_t st);

// ---- batched persistent screening ----------------------------------------------------
// A chunk is PMGB_THREADS insertions of one system: insertion block * n_per_block +
// chunk * PMGB_THREADS + tid.  Chunks of a system are numbered block-major from chunk_first;
// each has its own partial (and adjoint column) slot.  A work unit is a run of consecutive
// chunks of one block; a CTA keeps a framework that fits its ring resident across them.
struct BatchSystem {
    SysDev sys;
    long long n_per_block;
    int variant;          // template variant: index of (NS, charged), see pmgb_batch_variant
    int n_cols;           // adjoint columns (segments x template sites x 2), 0 without adjoint
    int chunk_first;      // first chunk slot of this system
    int ctas_per_block;   // chunks per insertion block
    long long col_base;   // adjoint: first of this system's chunk column partials (n_cols per chunk)
    long long out_base;   // adjoint: first of this system's 3 + n_cols combined outputs
    long long u_base;     // first of this system's insertions in the batch's per-insertion energies
    int img;              // forward run in spatial order: image lists over one order of the system's run
    int order_bits;       // image lists: Z-order cells per axis 2^order_bits (pmgb_run_order_bits)
    long long cell_base;  // image lists: first of this system's cells in the batch's order counts
};
struct BatchUnit {
    int system, block, chunk0, n_chunks;
};
struct BatchRun {
    unsigned long long seed;  // Philox key of system s: seed + s * 0x9E3779B97F4A7C15 (mod 2^64)
    double inv_temperature;
};
struct BatchArgs {
    const BatchSystem* systems;
    const BatchUnit* units;
    const int* order;         // processing order of the units
    int n_units;              // work units in the queue
    int* counter;             // work-queue head, zeroed before each run
    const BatchRun* run;      // device memory, so that a captured graph takes new seeds
    LsePartial* partials;     // [total chunks]
    unsigned int* status;
    // adjoint only
    float* dsum;              // per-CTA column scratch: [gridDim.x][max_cols][PMGB_THREADS]
    int max_cols;
    double* unit_cols;        // per-chunk weighted column sums, weights exp(-U/T - m_chunk)
    double* u;                // optional: per-insertion (U_vdw, U_es), system s at 2 * u_base
    // spatial order (optional): perm[u_base + block * n_per_block + slot] = insertion within the
    // block evaluated in that slot; the partials are then formed from u in insertion order
    const int* perm;
    double* unit_m;           // adjoint with perm: the max of -U/T of each processing chunk
    int no_resid;             // forward with FP64 refinement: no box-matrix residual (LaunchArgs)
};

// ---- FP64 refinement of the Boltzmann tail (pmgb_refine.cu) ---------------------------
struct RefineArgs {
    SysDev sys;                     // single-system mode
    const BatchSystem* systems;     // batch mode when non-null: chunk c belongs to system chunk_sys[c]
    const int* chunk_sys;
    const BatchRun* run;            // batch mode: seed and 1/T (device memory, for graph replays)
    int n_systems;                  // 1 in single-system mode
    long long n_per_block;          // single-system mode (batch: per system)
    int n_blocks, ctas_per_block;   // insertion i of block b: b * n_per_block + i; 256 per chunk
    unsigned long long seed;
    double inv_temperature;
    double tail;                    // weight fraction left unrefined per block (at most)
    double* block_out;              // [4 n_systems n_blocks] FP32-pass results, corrected in place
    double* u;                      // [2 n] per-insertion (U_vdw, U_es); refined entries replaced
    unsigned long long* hist;       // [n_systems * n_blocks * pmgb_refine_hist_words()]
    int* cut;                       // [n_systems * n_blocks]
    int* counts;                    // [chunks]
    int* offsets;                   // [chunks + 1]
    long long* list;                // [n] refined insertions (system << 40 | insertion), index order
    double* ref_u;                  // [3 n] their FP64 (U_vdw, U_sr, U_lr)
    int* counter;                   // [1] work counter of the chunked pass
    int* plan;                      // [n_systems + 1] first chunk-item of each system, then the total
    int* one_chunk;                 // [1] set when the chunk-items would exceed cap_items
    int* done;                      // [cap_entries] chunks finished per refined insertion
    double* part;                   // [4 cap_items] chunk partials (U_vdw, U_sr / coul, U_lr, overlap)
    LsePartial* partials;           // [chunks] the Widom pass's Boltzmann partials (re-formed where refined)
    long long cap_items, cap_entries;
    // where the entries' guest sites come from (REFINE_POSE_*): Widom poses, the caller's
    // explicit FP64 site coordinates, or energy-grid points of a single-site probe
    int pose_src;
    const double* site_xf;          // REFINE_POSE_SITES: [n x n_sites x 3] supercell fractions
    int grid_n[3], grid_rep[3];     // REFINE_POSE_GRID / _ROTGRID: points per axis, replication factors
    const double* grid_ax64;        // ... and the FP64 supercell fractions of the points along x, y, z (concatenated)
    long long point_base, item_base;  // REFINE_POSE_ROTGRID: block b at point point_base + b; rotation
                                      //   of insertion i from Philox counter item_base + i
};
// REFINE_POSE_ROTGRID: Widom insertions of a rotational energy grid (centre of mass at the block's
// grid point, Philox rotation)
enum RefinePose : int { REFINE_POSE_PHILOX = 0, REFINE_POSE_SITES = 1, REFINE_POSE_GRID = 2, REFINE_POSE_ROTGRID = 3 };
cudaError_t pmgb_launch_refine(const RefineArgs& a, int n_ctas, int n_sm, cudaStream_t st);
// Double-float energies of every explicit configuration 0..n-1 (n from *n_dev when n_dev is set,
// else n), written to a.ref_u as (U_vdw, U_es short-range, U_es long-range): pose_src
// REFINE_POSE_SITES; a.list, a.offsets (>= 1 entry), a.plan, a.done, a.part, a.counter scratch.
cudaError_t pmgb_launch_exact(const RefineArgs& a, long long n, const int* n_dev, int n_sm, cudaStream_t st);
// Re-evaluate in double-float every point of an FP32 energy grid whose error estimate (bound,
// from pmgb_launch_grid_bound) exceeds max(1e-5 |U|, 1e-4 K), and overwrite its value in grid
// (U * unit_factor): pose_src REFINE_POSE_GRID; a.counts / a.offsets hold one entry per 256
// points.  n_points = the grid's points.
cudaError_t pmgb_launch_grid_exact(const RefineArgs& a, const float* bound, float* grid, long long n_points,
                                   double unit_factor, int n_sm, cudaStream_t st);
// CTAs of the grid screen (one per PMGB_THREADS points)
int pmgb_grid_screen_ctas(long long n_points);
size_t pmgb_refine_hist_words();

// Index of the compiled template variant for n_sites guest sites with or without charges;
// -1 if there is none.
int pmgb_batch_variant(int n_sites, bool charged);

// kernels (defined in pmgb_kernels.cu); return cudaError_t of the launch
cudaError_t pmgb_launch_pairs(const LaunchArgs& a, int n_ctas, cudaStream_t st);
cudaError_t pmgb_launch_pairs_grad(const LaunchArgs& a, int n_ctas, cudaStream_t st);
// Energy grid of a single-site uncharged probe (POSE_GRID, OUT_GRID) plus each point's FP32
// error scale in a.bound_out (run_unit's BOUND form)
cudaError_t pmgb_launch_grid_bound(const LaunchArgs& a, int n_ctas, cudaStream_t st);
// The forward pass with the work it does counted into a.stats (run_unit's STATS form): guests of
// one or three sites; Widom poses take the centre-image form where the system does
cudaError_t pmgb_launch_pairs_stats(const LaunchArgs& a, int n_ctas, cudaStream_t st);
// persistent batch (defined in pmgb_batch.cu)
cudaError_t pmgb_batch_prepare(bool grad);  // function attributes, before any stream capture
cudaError_t pmgb_launch_batch(const BatchArgs& b, bool grad, int n_ctas, cudaStream_t st);
// per system: block_out[(s * n_blocks + b) * 4 ..] and, with grad, the combined columns
// out_cols[out_base ..] = (m, sum w, sum w U_es, sum w col_0, ...), w = exp(-U/T - m)
cudaError_t pmgb_launch_batch_reduce(const BatchSystem* systems, int n_systems, int n_blocks,
                                     const LsePartial* partials, const double* unit_cols, const double* unit_m,
                                     bool grad, double* block_out, double* out_cols, cudaStream_t st);
// Spatial order of every system's insertions (16^3 Z-order cells per (system, block)) and the
// insertion-order partials of a culled batch run; chunk_sys maps chunks to systems.
size_t pmgb_batch_order_cells();
cudaError_t pmgb_launch_batch_order(const BatchSystem* systems, const int* chunk_sys, int n_chunks, int n_systems,
                                    int n_blocks, const BatchRun* run, int* counts, int* perm, cudaStream_t st);
// Image-list systems of a batch: one order over each such system's run (cells: the batch's
// counts, system s at cell_base), perm[u_base + slot] = the system's insertion index.
cudaError_t pmgb_launch_batch_run_order(const BatchSystem* systems, const int* chunk_sys, int n_chunks, int n_systems,
                                        const BatchRun* run, int* cells, long long n_cells, int* perm, cudaStream_t st);
cudaError_t pmgb_launch_batch_lse(const BatchSystem* systems, const int* chunk_sys, int n_chunks, const BatchRun* run,
                                  const double* u, LsePartial* partials, cudaStream_t st);
cudaError_t pmgb_launch_reduce_blocks(const LsePartial* partials, int n_blocks, int ctas_per_block,
                                      double* block_out, cudaStream_t st);
// qxf: framework charge fractional coordinates (FP64, 3 per charge)
// S(k) of every k-vector from per-axis phasor tables e^{2 pi i h x_c}, |h| <= kmax[d]; `table`
// holds pmgb_structure_factor_table_len(n_q, kmax) entries of scratch
size_t pmgb_structure_factor_table_len(int n_q, const int kmax[3]);
cudaError_t pmgb_launch_structure_factor(const double* qxf, const double* q, int n_q,
                                         const int* kabc, const double* wt, int n_k, const int kmax[3],
                                         double2* table, double* sk_out, float2* skw_out, cudaStream_t st);
cudaError_t pmgb_launch_sample_poses(unsigned long long seed, long long start, long long n,
                                     float* xf_out, float* rot_out, cudaStream_t st);
cudaError_t pmgb_launch_philox(const unsigned int* ctr, const unsigned int* key, long long n,
                               unsigned int* out, cudaStream_t st);
cudaError_t pmgb_launch_fp32_peak(float* sink, int n_ctas, int iters, cudaStream_t st);
cudaError_t pmgb_launch_vdw_ordered(const double* f2c, int n_atoms, const double* atom_xf, const int* atom_sp,
                                    int n_sp, const double* eps, const double* sig2, double r2_cut, long long n_conf,
                                    int n_sites, const int* site_sp, const double* site_xf, double* out,
                                    cudaStream_t st);
cudaError_t pmgb_launch_rot_grid_out(const double* block_out, int n, double temperature, double log_n, double unit,
                                     float* out, cudaStream_t st);
cudaError_t pmgb_launch_bounded_wait_test(unsigned int* status, unsigned long long limit_ns, int arm,
                                          cudaStream_t st);
size_t pmgb_pairs_smem_bytes();

// the double-float phase table of the refinement's reciprocal space, built once per device
// (synchronously at context creation, before any launch or capture reads it)
cudaError_t pmgb_launch_phase_table(cudaStream_t st);

// record a failure message on ctx and return code (defined in pmgb_api.cu)
struct pmgb_ctx;
int pmgb_fail_message(pmgb_ctx* ctx, int code, const char* message);

// host set-up helpers (defined in pmgb_setup.cu)
struct PmgbSupercell {
    int32_t rep[3];
    double f_to_c[9];
    std::vector<double> atom_xf, charge_xf, charge_q;
    std::vector<int32_t> atom_species;
};
int pmgb_make_supercell(const double f_to_c[9], double r_cutoff, int32_t n_atoms, const double* atom_xf,
                        const int32_t* atom_species, int32_t n_charges, const double* charge_xf,
                        const double* charge_q, PmgbSupercell& sc, const char** why);
int pmgb_ewald_kvectors(const double f_to_c[9], double sr_cutoff, double precision, double* alpha_out,
                        double* max_k2_out, int32_t kreps_out[3], std::vector<int32_t>* abc, std::vector<double>* wt,
                        int64_t* n_k_out);

// fixed per-device scratch of pmgb_widom_noalloc (defined in pmgb_kernels.cu)
#define PMGB_NOALLOC_MAX_CTAS 65536   // LsePartial entries: 3 MiB, up to 16.7M insertions per call
#define PMGB_NOALLOC_MAX_DEVICES 64
cudaError_t pmgb_noalloc_scratch(int device, LsePartial** ptr);

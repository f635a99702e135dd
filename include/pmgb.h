/*
 * pmgb.h -- C ABI of libpmgb, the GB300 (sm_103a) implementation of the Widom-insertion
 * Henry-coefficient and potential-energy-grid path of PorousMaterials.jl.
 *
 * The reference (PorousMaterials.jl v0.4.2, pure Julia) has no FFI for this path; its
 * boundary is the exported Julia functions.  Each entry point below names the reference
 * function it replaces (file:line inside the PorousMaterials.jl source tree).  A Julia
 * package binds these with `ccall` (porousmaterials.jl_gb300/julia/PorousMaterialsGB300.jl);
 * Python binds them with ctypes (porousmaterials.jl_gb300/pmgb/_lib.py).
 *
 * Conventions
 *   - Every function returns PMGB_OK (0) or a negative PMGB_ERR_* code; the message of the
 *     last failure is available from pmgb_last_error().  Nothing aborts or throws.
 *   - 3x3 matrices are column-major (Julia layout): m[i + 3*j] = M[i][j].
 *   - Coordinate arrays are packed xyz triplets: xf[3*k + d].
 *   - Host buffers are owned by the caller; the library copies in and writes out.
 *     Device buffers are owned by the context / system handles.
 *   - A context is not thread-safe: use one context per host thread.  All work of a
 *     context runs in order on one CUDA stream.
 *   - Kernel-side failures (a bounded wait that gave up) are reported through a status
 *     word read back after each synchronous call (PMGB_ERR_DEVICE_STATUS); no kernel traps.
 */
#ifndef PMGB_H
#define PMGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PMGB_ABI_VERSION 1

#define PMGB_OK 0
#define PMGB_ERR_INVALID_ARGUMENT (-1)
#define PMGB_ERR_CUDA (-2)
#define PMGB_ERR_OUT_OF_MEMORY (-3)
#define PMGB_ERR_DEVICE_STATUS (-4)
#define PMGB_ERR_UNSUPPORTED (-5)
#define PMGB_ERR_NOT_READY (-6)

typedef struct pmgb_ctx pmgb_ctx;
typedef struct pmgb_system pmgb_system;

/* ---- library / context ---------------------------------------------------------- */

/* ABI version of the loaded library (PMGB_ABI_VERSION). */
int pmgb_abi_version(void);

/* Create a context on CUDA device `device` with its own stream.  No reference
 * counterpart: the reference runs in Julia worker processes (src/henry.jl:109).
 * Systems, move handles and batches keep what they use alive (a system its context, a move
 * handle its system, a batch its systems and context): handles may be destroyed in any order. */
int pmgb_create(int device, pmgb_ctx** out);
void pmgb_destroy(pmgb_ctx* ctx);

/* Message of the last failure on this context ("" if none); NULL ctx gives the last
 * failure of pmgb_create. */
const char* pmgb_last_error(const pmgb_ctx* ctx);

/* Run subsequent work on `stream` (a cudaStream_t); NULL restores the context's own stream.
 * Work already queued on the previous stream is waited for first: the context's device memory
 * comes from a stream-ordered pool, ordered on the context's current stream. */
int pmgb_set_stream(pmgb_ctx* ctx, void* stream);
int pmgb_synchronize(pmgb_ctx* ctx);

/* ---- system: replicated crystal + force field + guest molecule ---------------------
 *
 * Replaces the state the reference threads through its hot loop: the replicated
 * `Crystal` (src/henry.jl:80-89; Xtals.replicate), the `LJForceField` tables
 * (src/forcefield.jl:12-22, ϵ and σ² indexed by species) and the rigid `Molecule`
 * (src/molecule.jl:10-15, converted to fractional coordinates at src/henry.jl:89).
 *
 *   f_to_c            supercell box (columns = lattice vectors, Å)
 *   atom_xf/species   crystal.atoms: fractional coordinates of the supercell, species id
 *   charge_xf/q       crystal.charges: fractional coordinates, charges (e)
 *   epsilon, sigma2   n_species x n_species tables (K, Å²), species ids index both axes
 *                     (row-major and symmetric: epsilon[a*n_species + b])
 *   r2_cutoff         LJ cutoff radius squared (ljff.r²_cutoff)
 *   guest_atom_x      Cartesian offsets of the guest's LJ sites from its centre of mass
 *   guest_charge_x/q  Cartesian offsets and charges of the guest's point charges
 * Guest LJ sites and charges at the same offset are merged into one site; at most 8
 * sites result.  Electrostatics are on iff n_charges > 0 and n_guest_charges > 0
 * (src/henry.jl:93) and then need pmgb_system_set_ewald. */
int pmgb_system_create(pmgb_ctx* ctx, const double f_to_c[9],
                       int32_t n_atoms, const double* atom_xf, const int32_t* atom_species,
                       int32_t n_charges, const double* charge_xf, const double* charge_q,
                       int32_t n_species, const double* epsilon, const double* sigma2,
                       double r2_cutoff,
                       int32_t n_guest_atoms, const double* guest_atom_x,
                       const int32_t* guest_atom_species,
                       int32_t n_guest_charges, const double* guest_charge_x,
                       const double* guest_charge_q,
                       pmgb_system** out);

/* ---- host-side set-up from a unit cell (no device work) ----------------------------------
 * replication_factors(box, r_cutoff) (src/forcefield.jl:120-158): the smallest supercell whose
 * perpendicular half-widths reach r_cutoff.  f_to_c is the unit cell (column-major). */
int pmgb_replication_factors(const double f_to_c[9], double r_cutoff, int32_t rep_out[3]);

/* setup_Ewald_sum(box, sr_cutoff; ϵ=precision) (src/electrostatics.jl:256-272 with
 * determine_ewald_params :123-141, required_kreps :157-175, precompute_kvec_wts :198-232) for the
 * supercell box f_to_c: α, |k|²_max, kreps and the k-vectors (ka, kb, kc) with their weights, in
 * the reference's order.  The two precision conditions are solved by bisection on the reference's
 * brackets.  *n_kvecs_out always receives the number of k-vectors; they are written when capacity
 * holds them all (capacity 0: query the count only). */
int pmgb_ewald_setup(const double f_to_c[9], double sr_cutoff, double precision, int64_t capacity,
                     double* alpha_out, double* max_k2_out, int32_t kreps_out[3], int64_t* n_kvecs_out,
                     int32_t* kvec_abc, double* kvec_wt);

/* pmgb_system_create from the UNIT cell, with the rest of henry_coefficient's set-up done
 * natively (src/henry.jl:78-97): the replication factors for r_cutoff, the replicated supercell
 * (Xtals.replicate: images (i, j, k) with k fastest, coordinates (x + shift) / rep), and, when the
 * framework and the guest are both charged, the Ewald parameters at ewald_precision
 * (pmgb_ewald_setup) and pmgb_system_set_ewald.  The LJ cutoff is r_cutoff² and the short-range
 * Ewald cutoff r_cutoff, as the reference sets both from the force field.  repfactors_out
 * (optional) receives the replication.  Other arguments as pmgb_system_create. */
int pmgb_system_create_unitcell(pmgb_ctx* ctx, const double f_to_c[9],
                                int32_t n_atoms, const double* atom_xf, const int32_t* atom_species,
                                int32_t n_charges, const double* charge_xf, const double* charge_q,
                                int32_t n_species, const double* epsilon, const double* sigma2,
                                double r_cutoff,
                                int32_t n_guest_atoms, const double* guest_atom_x,
                                const int32_t* guest_atom_species,
                                int32_t n_guest_charges, const double* guest_charge_x,
                                const double* guest_charge_q, double ewald_precision,
                                int32_t repfactors_out[3], pmgb_system** out);

/* Many systems from their unit cells in one call: the set-up of a screen over frameworks (the
 * loop of src/henry.jl:78-97 over them).  System i is exactly what pmgb_system_create_unitcell
 * makes from entry i of every array argument (one count or pointer per system; species tables
 * n_species[i]^2 each).  The host work -- replication, records, Ewald parameters and k-vectors,
 * the choice of k-vectors once S(k) is known -- runs on n_threads host threads (0: one per
 * hardware thread, at most 64), and the device work is enqueued back to back through pinned
 * staging, with two stream synchronisations in all.  repfactors_out (optional) receives 3 per
 * system.  All or nothing: on failure no handle is created and the message names the system. */
int pmgb_systems_create_unitcell(pmgb_ctx* ctx, int32_t n_systems, const double* const* f_to_c,
                                 const int32_t* n_atoms, const double* const* atom_xf,
                                 const int32_t* const* atom_species, const int32_t* n_charges,
                                 const double* const* charge_xf, const double* const* charge_q,
                                 const int32_t* n_species, const double* const* epsilon,
                                 const double* const* sigma2, double r_cutoff, const int32_t* n_guest_atoms,
                                 const double* const* guest_atom_x, const int32_t* const* guest_atom_species,
                                 const int32_t* n_guest_charges, const double* const* guest_charge_x,
                                 const double* const* guest_charge_q, double ewald_precision, int32_t n_threads,
                                 int32_t* repfactors_out, pmgb_system** out);

/* Ewald parameters: EwaldParams (src/electrostatics.jl:54-63) as produced by
 * setup_Ewald_sum (src/electrostatics.jl:256-272): α, the short-range cutoff, and the
 * k-vectors (ka, kb, kc) with weights wt (precompute_kvec_wts, :198-232).  The
 * structure factor S(k) of the framework charges is built on the device here. */
int pmgb_system_set_ewald(pmgb_system* sys, double alpha, double sr_cutoff,
                          int32_t n_kvecs, const int32_t* kvec_abc, const double* kvec_wt);
void pmgb_system_destroy(pmgb_system* sys);

/* Sizes of the device-resident system: out[0..5] = (framework records incl. padding,
 * species segments, k-vectors given, k-vectors evaluated, guest sites, bytes copied
 * host->device when the system and its Ewald state were built).  Fewer k-vectors are
 * evaluated than given when the framework is a replicated cell: S(k) then vanishes for
 * every k that is not a multiple of the replication factors, and those are skipped.
 * No reference counterpart (diagnostics). */
int pmgb_system_info(const pmgb_system* sys, int64_t* out6);

/* Number of guest sites and, for each site, the guest atom / guest charge it carries
 * (-1 when none).  Explicit-coordinate calls take one position per site. */
int pmgb_system_n_sites(const pmgb_system* sys);
int pmgb_system_sites(const pmgb_system* sys, int32_t* site_atom, int32_t* site_charge);

/* S(k) = Σ_c q_c e^{ik·r_c} for each k-vector (re, im interleaved; 2*n_kvecs doubles).
 * The reference evaluates the same sum per guest charge in _ϕ
 * (src/electrostatics.jl:361-372); exposed for checking. */
int pmgb_structure_factor(pmgb_system* sys, double* sk_out);

/* ---- single-configuration energies --------------------------------------------------
 * For n_conf guest configurations given as fractional site coordinates of the supercell
 * (n_conf x n_sites x 3), out[3*i..3*i+2] = (U_vdw, U_es short-range, U_es long-range) in K.
 * Replaces vdw_energy(crystal, molecule, ljff) (src/vdw_energetics.jl:62-64 -> 25-47;
 * +Inf on overlap) and electrostatic_potential_energy(crystal, molecule, eparams, eikr)
 * (src/electrostatics.jl:331-342 -> _ϕ :347-388; the EwaldSum sr and lr parts).
 * With exact energies (pmgb_system_set_exact, the default) every configuration is evaluated in
 * double-float (~48-bit) arithmetic from its FP64 coordinates: within ~1e-10 relative of the
 * FP64 reference.  Off: the FP32 pair pass, within ~4e-6 of the sum of the terms' magnitudes. */
int pmgb_energies(pmgb_system* sys, int64_t n_conf, const double* site_xf, double* out);

/* Exact single-configuration energies for this system (default on): pmgb_energies,
 * pmgb_energies_grad (energies; gradients stay FP32), pmgb_move_* (handles created while on)
 * and the energy grids meet the reference's FP64 values to 1e-5 relative or 1e-4 K for every
 * configuration and grid point.  Grids run the FP32 pass with a per-point estimate of its
 * rounding error and re-evaluate in double-float the points whose estimate exceeds that
 * tolerance (or that have a pair within rounding of the cutoff or the overlap distance).
 * 0 switches it off (FP32 only).  No reference counterpart: the reference is FP64 throughout. */
int pmgb_system_set_exact(pmgb_system* sys, int32_t on);

/* ---- Widom insertions ----------------------------------------------------------------
 * Replaces the pmap over N_BLOCKS blocks of _conduct_Widom_insertions
 * (src/henry.jl:103-113 -> :185-265).  Insertion i (0 <= i < n_blocks*n_per_block)
 * belongs to block i / n_per_block; its pose is drawn from Philox4x32-10 keyed by
 * (seed, i): centre of mass uniform in the supercell, uniform random rotation.
 * block_out[4*b..4*b+3] = (log Σ e^{-U/T}, Σ U_vdw e^{-U/T} / Σ e^{-U/T},
 *                          Σ U_es e^{-U/T} / Σ e^{-U/T}, number of insertions with U = +Inf)
 * (the reference's boltzmann_factor_sum and wtd_energy_sum, henry.jl:205-244, in
 * log-sum-exp form).  u_out (optional, may be NULL) receives (U_vdw, U_es) per insertion. */
int pmgb_widom(pmgb_system* sys, int64_t n_per_block, int32_t n_blocks, uint64_t seed,
               double temperature, double* block_out, double* u_out);

/* FP64 refinement of the Boltzmann tail for this system's Widom runs (pmgb_widom,
 * pmgb_widom_device, pmgb_widom_adjoint; default off): after the FP32 pass, the insertions that
 * carry all but `tail_fraction` of each block's Boltzmann weight are re-evaluated in FP64 (LJ,
 * real-space erfc, reciprocal space on the FP64 S(k)) and the block results corrected, so that
 * log K_H is exact to tail_fraction x the FP32 error of the remainder.  Refined insertions
 * report their FP64 energies in u_out.  0 switches it off.  No reference counterpart: the
 * reference is FP64 throughout (src/henry.jl:212-244). */
int pmgb_system_set_refine(pmgb_system* sys, double tail_fraction);

/* Accessibility gate for this system's Widom runs (the accessibility_grid branch of
 * src/henry.jl:225 -> accessible, src/grid.jl:778-836): data is a Bool grid over the UNIT
 * cell, n_pts[0]*n_pts[1]*n_pts[2] bytes with i fastest (0 = inaccessible), repfactors the
 * replication of this system's supercell.  An insertion whose centre of mass, scaled into the
 * unit cell, has its nearest grid node and all 26 neighbours inaccessible gets U_vdw = U_es =
 * +Inf.  data = NULL removes the gate. */
int pmgb_system_set_accessibility(pmgb_system* sys, const int32_t n_pts[3], const int32_t repfactors[3],
                                  const uint8_t* data);

/* Spatially ordered evaluation (default on) for pmgb_widom / pmgb_widom_device and the energy
 * grid: insertions of each block are processed in Hilbert-curve order of their centre of mass
 * (grid points in 4 x 4 x 2 bricks), and a warp skips the pair terms of framework records
 * beyond the cutoff of all its items.  The skipped terms are exact zeros and the block sums are formed in
 * insertion order, so results are bit-identical with it on or off.  No reference counterpart. */
int pmgb_system_set_cull(pmgb_system* sys, int32_t on);

/* Centre-image distances (default on) for Widom insertions of a guest with several sites: where
 * every perpendicular width of the supercell is at least 2 (cutoff + the largest site distance
 * from the pose centre) + 0.1 A, each framework record's minimum-image displacement from the pose
 * centre is converted once and every site subtracts its offset.  The pairs inside the cutoff and
 * their images are the per-site minimum images, so results differ from the per-site form (on = 0)
 * by FP32 rounding only.  No reference counterpart; a batch takes the setting its systems have
 * when it is created. */
int pmgb_system_set_centre_image(pmgb_system* sys, int32_t on);

/* Image lists for the spatially ordered Widom pass (no reference counterpart).  mode 0: off;
 * 1 (the default): where the run's insertions are dense enough that a CTA's list is expected to
 * hold under 90% of the records and the run fills the GPU (at least two CTAs of 256 insertions
 * per SM), or, in a batch, under 140% of the records; 2: always where they apply.  They apply where culling is on, the
 * guest has one or three sites and every perpendicular width exceeds twice the larger cutoff.  The
 * insertions of a run are sorted once by position; each CTA (256 insertions) gathers the periodic
 * images of the framework records within (cutoff + the spread of its guest sites) of its sites'
 * centre, as double-float Cartesian offsets, into a shared-memory list, and its lanes take
 * distances from that list (pairs closer than 4 A with the offsets' residuals).  The energies are
 * the per-site form's to FP32 rounding, with the same error bound against FP64.  A batch runs
 * its systems that take image lists over the same insertion order as a single-system run, so its
 * results equal those of single-system runs that take the same form (mode 0 or 2 on both sides;
 * in mode 1 the batch's bar is higher). */
int pmgb_system_set_image_lists(pmgb_system* sys, int32_t mode);

/* *on_out = 1 when a forward Widom run of n_insertions insertions of this system takes image
 * lists (the mode, culling, the guest, the widths and the density all allow it), else 0. */
int pmgb_system_image_lists(const pmgb_system* sys, int64_t n_insertions, int32_t* on_out);

/* Index of cell (x, y, z) of a grid of 2^bits cells per axis along the Hilbert curve that orders
 * the insertions of the spatially ordered Widom runs (J. Skilling's construction); -1 when bits is
 * outside 1..10 or a coordinate outside the grid.  Host-side, no device work: the code the order
 * kernels run, for checks of the order.  No reference counterpart. */
int pmgb_hilbert_cell(uint32_t x, uint32_t y, uint32_t z, int32_t bits);

/* *on_out = 1 when Widom insertions of this system take the centre-image form (switched on, a
 * guest with several sites, and every width wide enough for the current cutoffs), else 0. */
int pmgb_system_centre_image(const pmgb_system* sys, int32_t* on_out);

/* *on_out = 1 when the system's guest has three sites with site 0 at the centre of mass and
 * sites 1 and 2 mirror images through it with equal charges (CO2 as the reference's data files
 * give it): the reciprocal-space sums of its forward passes then carry the phase factors of
 * site 1 alone, e^{-ik.d_2} = conj(e^{-ik.d_1}).  Else 0.  Results agree with the general form to
 * FP32 rounding; the FP64 refinement does not use the shortcut. */
int pmgb_system_kspace_mirror(const pmgb_system* sys, int32_t* on_out);

/* Number of items the system's last double-float pass re-evaluated (synchronises): insertions of
 * the last refined Widom run, configurations of the last exact pmgb_energies call, or points of
 * the last exact energy grid. */
int pmgb_system_refined_count(pmgb_system* sys, int64_t* count_out);

/* Same computation on device-resident outputs, enqueued on the context stream without
 * synchronising (block_out_dev: 4*n_blocks doubles, u_out_dev optional). */
int pmgb_widom_device(pmgb_system* sys, int64_t n_per_block, int32_t n_blocks, uint64_t seed,
                      double temperature, double* block_out_dev, double* u_out_dev);

/* Widom insertions for callers that cannot let the library allocate.  Some hosts cannot have
 * cudaMalloc / cudaFree called under them during a run: cudaFree synchronises the whole
 * device (a stall for a host that keeps other work in flight on the GPU), and a process whose
 * device memory is held by another framework's caching allocator may find none left.  This
 * call makes no allocation and no free: its per-CTA partial sums live in a fixed per-device
 * array (3 MiB, held by every GPU that loads the library until the process exits), sized for
 * at most 65,536 CTAs: n_blocks * ceil(n_per_block / 256) <= 65536, i.e. up to 16.7M
 * insertions per call; larger requests fail with PMGB_ERR_INVALID_ARGUMENT.
 * What it computes: the unordered FP32 pass (per-site distances) with the poses of
 * pmgb_widom_device.  Its energies and block results equal pmgb_widom_device's bit for bit where
 * that call takes per-site distances too (culling alone changes no result bit); where
 * pmgb_widom_device takes image lists (pmgb_system_set_image_lists) the two differ by FP32
 * rounding.
 * FP64 tail refinement needs per-run scratch, so a system with pmgb_system_set_refine(> 0) is
 * refused with PMGB_ERR_INVALID_ARGUMENT rather than given an unrefined K_H.
 * The caller passes device-resident outputs (block_out_dev: 4*n_blocks doubles, u_out_dev
 * optional).  The first call on a device looks up the array's device address (once per
 * device, cached; host threads may race on that first lookup harmlessly, all storing the same
 * address); make that first call before any stream capture.  All calls on a device share the
 * one array and overwrite it: calls that overlap on the GPU (other streams or threads) race
 * and must be serialised by the caller.  No counterpart in the reference. */
int pmgb_widom_noalloc(pmgb_system* sys, int64_t n_per_block, int32_t n_blocks, uint64_t seed,
                       double temperature, double* block_out_dev, double* u_out_dev);

/* Poses the Widom kernel uses for insertions start .. start+n-1: xf_out (n x 3, centre of
 * mass, supercell fractional) and rot_out (n x 9, column-major rotation applied to the
 * Cartesian site offsets).  Replaces rand(3) + random_rotation! (src/henry.jl:214-220,
 * src/molecule.jl:233-281). */
int pmgb_sample_poses(pmgb_ctx* ctx, uint64_t seed, int64_t start, int64_t n,
                      float* xf_out, float* rot_out);

/* ---- adjoint (no reference counterpart: the reference has no derivatives) ------------------
 * Widom insertions as pmgb_widom plus the Boltzmann-weighted parameter derivatives, recomputing
 * every pair term instead of storing it.  With w_i = exp(-U_i/T - M), M = dtheta[0]:
 *   dtheta[0] = M (= max_b block_out[4b]),  dtheta[1] = Σ_i w_i,  dtheta[2] = Σ_i w_i U_es,i,
 *   dtheta[3 + 2(a*n_species + b)]     = Σ_i w_i ∂U_i/∂ε_ab,
 *   dtheta[3 + 2(a*n_species + b) + 1] = Σ_i w_i ∂U_i/∂σ²_ab   (a: guest species, b: framework).
 * dK_H/dθ = -e^M Σ_i w_i ∂U_i/∂θ / (T · R T n_per_block · n_blocks) for the block-mean K_H of
 * src/henry.jl:120,141; ∂U_es/∂λ = U_es for framework charges scaled by λ.  grad_out (optional,
 * n x 3 floats) receives dU/dx of each insertion's centre of mass (K/Å; the force is minus it).
 * The (a, b) derivatives of a symmetric table entry used in both orders add. */
int pmgb_widom_adjoint(pmgb_system* sys, int64_t n_per_block, int32_t n_blocks, uint64_t seed,
                       double temperature, double* block_out, double* dtheta, double* u_out,
                       float* grad_out);

/* ---- Monte Carlo moves (guest-host energy of a few configurations at low latency) ------
 * The guest-host part of the energy a GCMC move needs (src/gcmc.jl:111-124 -> vdw_energy,
 * src/vdw_energetics.jl:62-64; plus the Ewald terms when the system is charged), as
 * pmgb_energies computes it, through a CUDA graph captured once: pinned staging, copy in,
 * one CTA per configuration with the framework split over its threads (FP32), or the
 * double-float pass when the system had exact energies on at creation, copy out.  A handle
 * serves 1..max_conf configurations per call; calls are synchronous. */
typedef struct pmgb_move pmgb_move;
int pmgb_move_create(pmgb_system* sys, int32_t max_conf, pmgb_move** out);
int pmgb_move_energies(pmgb_move* move, int32_t n_conf, const double* site_xf, double* out);
void pmgb_move_destroy(pmgb_move* move);

/* pmgb_energies plus dU/dx of the configuration's reference point (all sites moved rigidly;
 * grad_out: n_conf x 3 floats, K/Å).  The energies follow pmgb_system_set_exact; the
 * gradients come from the FP32 pass. */
int pmgb_energies_grad(pmgb_system* sys, int64_t n_conf, const double* site_xf, double* out,
                       float* grad_out);

/* ---- energy grid -----------------------------------------------------------------------
 * Replaces energy_grid(crystal, molecule, ljff; resolution=(n1,n2,n3)) for single-site
 * probes (src/grid.jl:291-362): point (i,j,k) sits at (i/(n1-1), j/(n2-1), k/(n3-1)) of
 * the unit cell, i.e. that divided by repfactors in the supercell this system holds;
 * out[i + n1*(j + n2*k)] = U_vdw * unit_factor (1 for K, 8.314/1000 for kJ/mol), rounded to
 * FP32; with exact energies (pmgb_system_set_exact) every value meets the FP64 reference to
 * 1e-5 relative or 1e-4 K before that rounding. */
int pmgb_energy_grid(pmgb_system* sys, const int32_t n_pts[3], const int32_t repfactors[3],
                     double unit_factor, float* out);
int pmgb_energy_grid_device(pmgb_system* sys, const int32_t n_pts[3], const int32_t repfactors[3],
                            double unit_factor, float* out_dev);

/* Rotational energy grid: energy_grid's branch for probes that need rotations (several sites
 * or charges; src/grid.jl:338-351).  At each point (placed as in pmgb_energy_grid) the probe's
 * centre of mass takes n_rotations uniform random orientations -- orientation r of point p
 * from Philox4x32-10 keyed by seed at counter p * n_rotations + r, as pmgb_sample_poses draws
 * them -- and out[p] = -T log(Σ_r e^{-U_r/T} / n_rotations) * unit_factor, with U = U_vdw plus
 * the Ewald energy when crystal and probe are charged (+Inf where every orientation overlaps).
 * With exact energies (pmgb_system_set_exact) or tail refinement on, the orientations that carry
 * all but 1e-3 (or the system's refinement fraction) of each point's Boltzmann weight are
 * re-evaluated in FP64.  The reference's own branch passes a Frac molecule to the one-argument
 * random_rotation!, which its v0.4.2 does not define (src/molecule.jl:269 takes a box). */
int pmgb_energy_grid_rotational(pmgb_system* sys, const int32_t n_pts[3], const int32_t repfactors[3],
                                int32_t n_rotations, double temperature, uint64_t seed, double unit_factor,
                                float* out);

/* Energy grid plus its adjoint: grad_out (optional, 3 floats per point) = dU/dr at each point
 * (K/Å, Cartesian), and dtheta as for pmgb_widom_adjoint with the grid points as the samples
 * (w_p = exp(-U_p/T - M), M = max_p -U_p/T): the grid estimate
 * K_H,grid = Σ_p e^{-U_p/T} / (R T n_points) has dK/dθ = -e^M Σ_p w_p ∂U_p/∂θ / (T R T n_points).
 * The grid values follow pmgb_system_set_exact; the weights and gradients use the FP32 pass. */
int pmgb_energy_grid_adjoint(pmgb_system* sys, const int32_t n_pts[3], const int32_t repfactors[3],
                             double unit_factor, double temperature, float* out, float* grad_out,
                             double* dtheta);

/* ---- batched screening (no reference counterpart: henry_coefficient takes one framework
 * per call, src/henry.jl:34) ---------------------------------------------------------------
 * Widom insertions for many systems (each its own framework and guest, of any size) in one
 * persistent kernel launch, captured once in a CUDA graph and replayed.  System s runs
 * n_blocks blocks of n_per_block[s] insertions with Philox key seed + s * 0x9E3779B97F4A7C15
 * (mod 2^64): the insertions, energies and block results of pmgb_widom with that seed.
 * with_adjoint adds the Boltzmann-weighted parameter sums of pmgb_widom_adjoint (dtheta),
 * accumulated inside the launch with weights relative to M = max_i -U_i/T of each system.
 * All systems must belong to ctx; the batch holds them (destroying a system handle first is fine). */
typedef struct pmgb_batch pmgb_batch;
int pmgb_batch_create(pmgb_ctx* ctx, int32_t n_systems, pmgb_system* const* systems,
                      const int64_t* n_per_block, int32_t n_blocks, int32_t with_adjoint,
                      pmgb_batch** out);
void pmgb_batch_destroy(pmgb_batch* batch);

/* Launch shape: n_ctas resident CTAs pulling work units (0 = two per SM, the maximum), the
 * unit order (0: estimated cost, largest first; 1: system by system) and the insertion tile
 * of a unit: runs of 256-insertion chunks of one block worth about unit_mflop MFLOP, over
 * which a framework that fits the shared-memory ring stays resident (0: one chunk per unit).
 * Re-captures the graph; results of earlier runs are no longer available. */
int pmgb_batch_configure(pmgb_batch* batch, int32_t n_ctas, int32_t order, double unit_mflop);

/* Autotuner: times candidate launch shapes (unit work 0/32/128/512 MFLOP, then 1 or 1.5 or 2
 * CTAs per SM, then unit order) over `repeats` graph replays each with CUDA events, keeps the
 * fastest and returns its ms per run. */
int pmgb_batch_tune(pmgb_batch* batch, uint64_t seed, double temperature, int32_t repeats,
                    double* best_ms_out);

/* FP64 refinement of the Boltzmann tail of every system's blocks, as pmgb_system_set_refine
 * (0: off, the default).  Allocates per-insertion scratch on first use and re-captures the graph. */
int pmgb_batch_set_refine(pmgb_batch* batch, double tail_fraction);

/* Spatially ordered processing with cutoff culling, as pmgb_system_set_cull (on by default):
 * each (system, block)'s insertions are sorted into 16^3 cells of the unit cell, ordered along a
 * Hilbert curve, and block results are formed from the per-insertion energies in insertion order, so they equal
 * those of an unordered run bit for bit.  Allocates scratch on first use and re-captures. */
int pmgb_batch_set_cull(pmgb_batch* batch, int32_t on);

/* Insertions of each system the last run re-evaluated in FP64 (n_systems values; synchronises). */
int pmgb_batch_refined_counts(pmgb_batch* batch, int64_t* per_system);

/* Per-insertion (U_vdw, U_es) in K of the last run, system after system, each system's insertions
 * in index order (block-major), the refined insertions with their FP64 energies: 2 * total
 * insertions doubles (synchronises).  Available when the batch culls or refines (both keep every
 * insertion's energy); PMGB_ERR_NOT_READY otherwise or before the first run.  No reference
 * counterpart (the per-insertion energies of _conduct_Widom_insertions, henry.jl:214-233). */
int pmgb_batch_energies(pmgb_batch* batch, double* u_out);

/* Enqueue one run (one graph replay) on the context stream; does not synchronise. */
int pmgb_batch_launch(pmgb_batch* batch, uint64_t seed, double temperature);

/* Wait for the last run and copy out its results: block_out[(s*n_blocks + b)*4 ..] as
 * pmgb_widom's, and with the adjoint dtheta: per system, in order, 3 + 2*n_species(s)^2
 * doubles laid out as pmgb_widom_adjoint's (dtheta may be NULL without the adjoint). */
int pmgb_batch_results(pmgb_batch* batch, double* block_out, double* dtheta);

/* out8 = (work units, n_ctas, order, dtheta length, device bytes held, insertions per run,
 *         256-insertion chunks, unit MFLOP target). */
int pmgb_batch_info(const pmgb_batch* batch, int64_t* out8);

/* ---- utilities -------------------------------------------------------------------------- */

/* Philox4x32-10 of n (counter[4], key[2]) pairs, for checking the generator bit for bit. */
int pmgb_philox4x32_10(pmgb_ctx* ctx, int64_t n, const uint32_t* ctr, const uint32_t* key,
                       uint32_t* out);

/* Guest-host van der Waals energies in FP64 in the reference's own operation order:
 * vdw_energy(atoms_i, atoms_j, box, ljff) (src/vdw_energetics.jl:25-47), with Xtals'
 * nearest_image! (d -= sign(d) where |d| > 1/2) and the f_to_c product summed left to right,
 * every operation rounded separately (no fused multiply-adds), the atoms summed in the order
 * given.  Configurations whose energies are equal in exact arithmetic (inversion images on a
 * grid) then compare as the reference's FP64 arithmetic compares them; find_energy_minimum_gridsearch
 * (src/energy_min.jl:75-85) takes its argmin over these values.  One thread per configuration,
 * serial in the atoms: meant for a few configurations.
 *   f_to_c:   the (replicated) box, column-major as everywhere in this header
 *   atom_xf:  n_atoms x 3 fractional coordinates, in the crystal's atom order
 *   eps, sigma2: n_species x n_species, row = guest site species, column = atom species
 *   site_xf:  n_conf x n_sites x 3 fractional guest site coordinates
 *   out:      n_conf energies in K (+Inf where a pair is closer than r^2 = 0.1 A^2) */
int pmgb_vdw_energy_ordered(pmgb_ctx* ctx, const double f_to_c[9], int32_t n_atoms, const double* atom_xf,
                            const int32_t* atom_species, int32_t n_species, const double* eps,
                            const double* sigma2, double r2_cutoff, int64_t n_conf, int32_t n_sites,
                            const int32_t* site_species, const double* site_xf, double* out);

/* FP32 FMA throughput probe: runs n_ctas x 256 threads x iters x 128 FMAs and returns the
 * measured TFLOP/s (the roofline denominator of the pair kernels). */
int pmgb_fp32_peak(pmgb_ctx* ctx, int n_ctas, int iters, double* tflops_out);

/* Read and clear the device status word (0 = no kernel-side failure). */
int pmgb_device_status(pmgb_ctx* ctx, uint32_t* status_out);

/* Self-test of the failure path of the kernels' bounded waits (no reference counterpart): one
 * thread waits at most limit_ns (1 .. 1e8) on a shared-memory mbarrier.  arm = 1 announces a
 * transfer that nothing delivers (no copy is issued, so none is in flight when the wait gives
 * up): the kernel records the staging-timeout bit in the status word and returns, and the call
 * returns PMGB_ERR_DEVICE_STATUS with the status cleared.  arm = 0 completes the phase: PMGB_OK. */
int pmgb_test_bounded_wait(pmgb_ctx* ctx, int64_t limit_ns, int32_t arm);

/* Work counts (no reference counterpart; measurement of the counted-work roofline): the forward
 * pass of pmgb_widom_device (spatially ordered, with its cutoff culling; the FP32 pass, no
 * refinement) or of pmgb_energy_grid (its FP32 pass), run with counters:
 * counts_out = (guest-site-to-record distances evaluated -- the records of sub-chunks skipped whole
 * are not -- , LJ pair terms inside the LJ cutoff, real-space pair terms inside the short-range
 * cutoff).  Results are not returned.  Guests of one or three sites. */
int pmgb_widom_work_counts(pmgb_system* sys, int64_t n_per_block, int32_t n_blocks, uint64_t seed,
                           int64_t counts_out[3]);
int pmgb_energy_grid_work_counts(pmgb_system* sys, const int32_t n_pts[3], const int32_t repfactors[3],
                                 int64_t counts_out[3]);

/* Kernel timing (no reference counterpart; measurement): while on, every Widom pass records a
 * CUDA event before and after its pair-kernel launch on the launching stream (at most 4096
 * launches between two reads).  pmgb_kernel_timing synchronises on the recorded events and
 * returns their summed duration (ms) and count since the last read, then clears them. */
int pmgb_set_kernel_timing(pmgb_ctx* ctx, int32_t on);
int pmgb_kernel_timing(pmgb_ctx* ctx, double* total_ms, int64_t* launches);

#ifdef __cplusplus
}
#endif
#endif /* PMGB_H */

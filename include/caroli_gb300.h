/* caroli_gb300 — C ABI of the GB300 (sm_103a) nested-dissection transport of caroli.
 *
 * This is the boundary a caroli caller binds: plain pointers and sizes, an int status on every
 * call, no exceptions across the ABI. The caller owns its host buffers; the library owns the
 * device memory. One CUDA stream per context. Thread-safe per context: every call taking a context
 * holds the context's lock for its whole duration, so threads sharing a context are serialised
 * (caroli_ctx_destroy waits for a call in progress; none may start after it). Contexts are
 * independent of each other.
 *
 * Reference interfaces each entry point replaces (caroli, crates/caroli-green/src/nested.rs):
 *   caroli_ctx_create / caroli_ctx_destroy   the "cuda" feature's device handle, CudaDevice::new
 *                                            (crates/caroli-gpu/src/cuda.rs:162-183)
 *   caroli_plan_upload                       NestedTwoTerminal::from_model        nested.rs:530-610
 *   caroli_values_upload                     the H values of each disorder configuration
 *                                            (caroli-cli/src/run.rs:118-121 builds one system each)
 *   caroli_sigma_upload                      LeadSelfEnergies from self_energies  nested.rs:439-459, :652-676
 *   caroli_solve_batch                       transmission_with / transmission_with_precision /
 *                                            transmissions                        nested.rs:618-713
 *   caroli_scattering_states                 NestedTwoTerminal::scattering_states nested.rs:851-899
 *   caroli_lead_modes, caroli_sigma_from_modes  self_energies with a Hermitian definite lead coupling
 *                                            (DefiniteCoupling, modes.rs:514-713), Σ formed on the GPU
 *   caroli_values_generate                   the CLI's per-configuration disorder  caroli-cli/src/build.rs:251-310
 *   caroli_values_download                   (reads the generated values back)
 *   caroli_multi_leads                       NestedMultiTerminal::from_model      nested_multi.rs:61-153
 *   caroli_multi_sigma_upload                its self_energies                    nested_multi.rs:188-199
 *   caroli_multi_transmissions               transmissions_with_precision         nested_multi.rs:171-186
 *   caroli_multi_scattering_states           its scattering_states                nested_multi.rs:382-438
 *   caroli_multi_sector_transmissions        its sector_transmissions             nested_multi.rs:226-295
 *   caroli_transmission_matrix               transmission_eigenvalues / fano_factor nested.rs:753-780
 *   caroli_root_green                        lead_green / the root of smatrix     nested.rs:717-802
 *   caroli_transmission_with_grad            no counterpart: the reference has no derivative code;
 *   caroli_derivs_upload                     the adjoint of transmission_with (dT/dV, dT/dJ)
 *   caroli_gamma_override                    the thesis' Re Γ trace               caroli-validation/src/thesis.rs:84-95
 *   caroli_solve_multi, caroli_solve_batch_noalloc, caroli_set_*, caroli_last_*, caroli_region_*,
 *   caroli_kernel_*, caroli_probe_kernel     no counterpart: batching across systems, an
 *                                            allocation-free FP64 entry, controls and accounting
 *   caroli_last_error                        GreenError / GpuError text           caroli-green/src/lib.rs:34-47
 */
#ifndef CAROLI_GB300_H
#define CAROLI_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct caroli_ctx caroli_ctx;

/* Status codes: return values of every call, and per-solve statuses of caroli_solve_batch. */
enum {
  CAROLI_OK = 0,
  CAROLI_PIVOT_DELAYED = 1,   /* a front refused its pivots: caroli_solve_batch re-plans such solves
                                 with the front delayed (never returned there);
                                 caroli_solve_batch_noalloc returns it for the instance (re-solve it
                                 with caroli_solve_batch) */
  CAROLI_SINGULAR = 2,        /* GreenError::Singular: the root solve is singular or not finite */
  CAROLI_NONFINITE = 3,       /* T is not finite */
  CAROLI_REFINE_STALLED = 4,  /* mixed precision: refinement did not reach its tolerance */
  CAROLI_TIMEOUT = 5,         /* a bounded device wait ran out (caroli_set_wait_limit) */
  CAROLI_EINVAL = 16,         /* bad argument (message in caroli_last_error) */
  CAROLI_ENOMEM = 17,         /* device allocation failed */
  CAROLI_ECUDA = 18,          /* CUDA error (message in caroli_last_error) */
  CAROLI_EUNAVAILABLE = 19    /* no usable GPU (GpuError::Unavailable) */
};

/* Precision of the fronts below the root (Precision, caroli-green/src/precision.rs:22-32). */
enum {
  CAROLI_DOUBLE = 0, /* complex f64 throughout */
  CAROLI_SINGLE = 1, /* complex f32 fronts, f64 root and trace, unrefined (Precision::Single) */
  CAROLI_MIXED = 2   /* complex f32 fronts as a preconditioner of FP64 iterative refinement of the
                        whole solve (no counterpart; Precision gains a Mixed variant). Block solves
                        whose right lead has more than caroli_set_mixed_max_channels open
                        channels (one refinement right-hand side each) take the FP64 path. */
};

int caroli_ctx_create(int device_ordinal, caroli_ctx** out);
void caroli_ctx_destroy(caroli_ctx* ctx);
/* Message of the last failed call on `ctx`; with NULL, why the last caroli_ctx_create failed. */
const char* caroli_last_error(const caroli_ctx* ctx);

/* Two-terminal system (NestedTwoTerminal::from_model). All arrays are copied.
 *   n, row_ptr[n+1], cols[nnz]           CSR pattern of H (u32 columns, sorted per row)
 *   nsites, dim, cells[3*nsites]         site cells (first axis slowest), lattice dimension
 *   site_offsets[nsites], site_orbitals[nsites]
 *   range[3]                             hopping range per axis (>= 1)
 *   n_interior, interior[]               sites of the elimination tree (all but the two lead slices)
 *   nblocks, labels[n]                   independent block of each orbital, -1 for none
 *   left_ptr[nblocks+1], left[]          per block, device orbitals of the first slice (lead-cell order)
 *   right_ptr[nblocks+1], right[]        per block, device orbitals of the last slice
 * On success *plan_id identifies the system in later calls. */
int caroli_plan_upload(caroli_ctx* ctx, int64_t n, const int64_t* row_ptr, const uint32_t* cols, int64_t nsites,
                       int dim, const int64_t* cells, const int64_t* site_offsets, const int64_t* site_orbitals,
                       const int64_t* range, int64_t n_interior, const int64_t* interior, int nblocks,
                       const int32_t* labels, const int64_t* left_ptr, const int64_t* left,
                       const int64_t* right_ptr, const int64_t* right, int* plan_id);

/* Shape of a plan: blocks, tree fronts of block `block`, largest front, root size. */
int caroli_plan_info(caroli_ctx* ctx, int plan_id, int block, int64_t* fronts, int64_t* max_n, int64_t* max_ne,
                     int64_t* root_n, int64_t* arena_elems);

/* The tree fronts of a block in post-order (up to `capacity`; *count = all): variables n, variables
 * eliminated ne, execution level (children run at lower levels). No device work. */
int caroli_plan_fronts(caroli_ctx* ctx, int plan_id, int block, int64_t capacity, int32_t* n, int32_t* ne,
                       int32_t* level, int64_t* count);

/* H values of `nconfigs` disorder configurations on the plan's pattern: values[c*nnz + q] as
 * interleaved complex128 (re, im). Replaces previously uploaded values. */
int caroli_values_upload(caroli_ctx* ctx, int plan_id, int nconfigs, const double* values);

/* On-device disorder: the H values of `nconfigs` configurations generated on the GPU (no host
 * model build, no values upload), bit for bit the CLI's [[disorder]] entries
 * (caroli-cli/src/build.rs:251-310; caroli-disorder/src/{rng,lib}.rs). Configuration c of the
 * result is configuration first_config + c of the sequence: entry e draws from xoshiro256**
 * seed_from_u64(seed_e + first_config + c) (the CLI's seed_e is 1 + 1000 e unless the entry sets
 * one). Values = clean_values (interleaved complex128 on the plan's pattern) plus, on each site's
 * on-site block, every entry's term in order:
 *   CAROLI_ANDERSON  w (u - 1/2) on the diagonal of every site, sites in region order;
 *   CAROLI_MAGNETIC  floor(concentration * nsites) impurity sites (partial Fisher-Yates), a unit
 *                    moment each (CAROLI_MOMENTS_ISOTROPIC; _POLARIZED, moment_param = m_z; _CONE,
 *                    moment_param = -(1 - cos θ0)), and J (n_x S_x + n_y S_y + n_z S_z) on the
 *                    site, spin = S_x, S_y, S_z (orbitals x orbitals column-major complex128 each).
 * The pattern must hold every on-site entry a term can make non-zero (CAROLI_EINVAL otherwise).
 * Products and sums are rounded as the host rounds them: the values equal the host-built ones
 * exactly, except that the azimuth's cos and sin (isotropic and cone moments) may differ from the
 * host's libm in the last bit. Replaces the uploaded values. */
enum { CAROLI_ANDERSON = 0, CAROLI_MAGNETIC = 1 };
enum { CAROLI_MOMENTS_ISOTROPIC = 0, CAROLI_MOMENTS_POLARIZED = 1, CAROLI_MOMENTS_CONE = 2 };
typedef struct caroli_disorder {
  int32_t kind;           /* CAROLI_ANDERSON or CAROLI_MAGNETIC */
  int32_t moments;        /* CAROLI_MOMENTS_* (magnetic) */
  uint64_t seed;          /* configuration c draws from seed_from_u64(seed + c) */
  double strength;        /* Anderson w */
  double concentration;   /* magnetic: impurities per site */
  double exchange;        /* magnetic: J */
  double moment_param;    /* m_z (polarized) or -(1 - cos θ0) (cone) */
  int32_t orbitals;       /* magnetic: orbitals of every site (size of the spin matrices) */
  int32_t pad;
  const double* spin;     /* magnetic: S_x, S_y, S_z */
} caroli_disorder;
int caroli_values_generate(caroli_ctx* ctx, int plan_id, const double* clean_values, int nentries,
                           const caroli_disorder* entries, int nconfigs, int first_config);
/* The values of configuration `config` (nnz interleaved complex128) as the device holds them. */
int caroli_values_download(caroli_ctx* ctx, int plan_id, int config, double* values);

/* Lead self-energies of energy slot `slot` (any slot number; re-uploading replaces it):
 * sigma_l[b], sigma_r[b] are column-major complex128 (nl_b x nl_b, nr_b x nr_b) of block b.
 * w_right[b] (nr_b x channels[b], column-major complex128) with w_right w_right^† = Γ_R =
 * i(Σ_R - Σ_R^†) is the right-hand side of CAROLI_MIXED (gamma_root, nested.rs:1036-1047: the
 * eigenvectors of Γ_R with positive eigenvalues, scaled by their square roots). Both may be NULL:
 * the library then factors Γ_R by pivoted Cholesky, which is less robust when Σ_R is inexact
 * (Γ_R slightly indefinite). */
int caroli_sigma_upload(caroli_ctx* ctx, int plan_id, int slot, double energy, const double* const* sigma_l,
                        const double* const* sigma_r, const double* const* w_right, const int32_t* channels);

/* Self-energies formed on the GPU for leads with a Hermitian definite coupling H1 = s c 1 (square
 * and cubic leads; the fast path of modes.rs:540-710, "P = c 1": the eigenvectors Y of the cell
 * Hamiltonian serve every energy).
 * caroli_lead_modes: once per block and side (0 left, 1 right), Y (n x n column-major complex128,
 * n = the slice's orbitals in lead-cell order) and sc = s c.
 * caroli_sigma_from_modes: one energy into slot `slot`, from the per-mode roots the caller
 * classified (O(n) scalar work, modes.rs:641-668): d_left[b] = 1/λ_L and d_right[b] = λ_R (n
 * complex128 each), and the right lead's open channels (channel_modes[b], channels[b] of them, with
 * weights sqrt(-2 s c Im λ_R)). On the device: Σ_R = sc Y diag(λ_R) Y^†, Σ_L = sc Y diag(1/λ_L) Y^†
 * (FP64), Γ = i (Σ - Σ^†), and W_R = Y[:, channel_modes] diag(weights) with W_R W_R^† = Γ_R: what
 * caroli_sigma_upload would receive, without the host products, the eigendecomposition of Γ_R and
 * the copies. */
int caroli_lead_modes(caroli_ctx* ctx, int plan_id, int block, int side, int n, const double* y, double sc);
int caroli_sigma_from_modes(caroli_ctx* ctx, int plan_id, int slot, double energy, const double* const* d_left,
                            const double* const* d_right, const int32_t* channels, const int32_t* const* channel_modes,
                            const double* const* channel_weights);

/* Replaces the broadenings Γ_L, Γ_R of a slot's trace (after caroli_sigma_upload; NULL keeps a
 * block's), e.g. by their element-wise real part, the convention of the thesis codes
 * (caroli-validation/src/thesis.rs:84-95) that reproduce their published conductances. Affects the
 * CAROLI_DOUBLE and CAROLI_SINGLE traces. */
int caroli_gamma_override(caroli_ctx* ctx, int plan_id, int slot, const double* const* gamma_l,
                          const double* const* gamma_r);

/* T for `count` instances (energy slot, configuration), summed over the blocks.
 *   precision       CAROLI_DOUBLE, CAROLI_SINGLE or CAROLI_MIXED
 *   t[count]        transmissions; status[count] per-instance status (CAROLI_OK ...)
 *   err[count]      (may be NULL) error estimate: CAROLI_MIXED, the last refinement correction of
 *                   T; otherwise 0
 * Returns CAROLI_OK when the batch ran (individual solves may still carry a non-OK status). */
int caroli_solve_batch(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots, const int32_t* configs,
                       int precision, double* t, int32_t* status, double* err);

/* The double-precision transmission of caroli_solve_batch without any device allocation: no
 * counterpart in the reference. For callers that cannot allocate device memory while they solve
 * (a host program whose device memory another allocator has already reserved, or a loop where
 * allocation is not allowed). Every front, flag and work array of the call is carved from one
 * static device array of 64 MiB that each GPU loading this library keeps until the process exits;
 * a batch needing more is rejected with CAROLI_EINVAL and the size in caroli_last_error (solve
 * fewer instances per call). The system, its values and self-energies must have been uploaded
 * (those calls allocate). caroli_ctx_create looks the array's device address up once, with the
 * context's device current, so a call here makes only kernel launches and copies. Calls share the
 * array and run on the context's stream: calls that overlap on the GPU (other contexts, whose
 * streams are not ordered with this one) race. Fronts that refuse their pivots are not re-planned
 * here: those instances get CAROLI_PIVOT_DELAYED (use caroli_solve_batch for them). */
int caroli_solve_batch_noalloc(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots, const int32_t* configs,
                               double* t, int32_t* status);

/* Timed region on the context's stream: caroli_region_end returns the device time between the
 * two calls (CUDA events on the stream every kernel of the library runs on) and the number of
 * kernels the library launched in between. */
int caroli_region_begin(caroli_ctx* ctx);
int caroli_region_end(caroli_ctx* ctx, double* device_ms, int64_t* launches);

/* Per-kernel-class accounting (classes 0 .. caroli_kernel_classes()-1, named by
 * caroli_kernel_class_name): launches, algorithmic flops (complex multiply-add = 8 flops, the
 * reference's LU/TRSM/GEMM counts) and bytes attributed to the class. caroli_probe_kernel(ctx, k)
 * makes later solves time every launch of class k with CUDA events (-1: none); `ms` is their total.
 * `reset` clears the class's counters after reading them. */
int caroli_kernel_classes(void);
const char* caroli_kernel_class_name(int kclass);
int caroli_probe_kernel(caroli_ctx* ctx, int kclass);
int caroli_kernel_stats(caroli_ctx* ctx, int kclass, int64_t* launches, double* flops, double* bytes, double* ms,
                        int reset);

/* Derivatives of H with respect to `nparams` parameters (e.g. the exchange coupling J), per
 * configuration: values[(c * nparams + k) * nnz + q] as interleaved complex128 on the plan's
 * pattern. Used by caroli_transmission_with_grad for dT/dp. */
int caroli_derivs_upload(caroli_ctx* ctx, int plan_id, int nparams, const double* values);

/* T and its gradient (no counterpart in the reference, which has no derivative code): the adjoint
 * of transmission_with (nested.rs:682). For every instance, dt_dv[i * n + a] = dT/dV_a for the
 * on-site potential V_a of each orbital a (H -> H + V_a e_a e_a^T; 0 outside the blocks), and
 * dt_dp[i * nparams + k] = dT/dp_k for the uploaded derivatives (dt_dp may be NULL). Runs the
 * mixed path: one factorization, the forward solve X = G e_R W_R and one adjoint solve
 * Z = G^† Γ_L X with the same factors, both refined in FP64; dT/dV_a = 2 Re Σ_j X_aj conj(Z_aj),
 * dT/dp = 2 Re Σ_j Z_j^† (dH/dp) X_j. */
int caroli_transmission_with_grad(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots, const int32_t* configs,
                                  double* t, int32_t* status, double* dt_dv, double* dt_dp);

/* Scattering states ψ_p = G W_p on every device orbital (NestedTwoTerminal::scattering_states,
 * nested.rs:851-899) for `count` instances (energy slot, configuration). The caller supplies the
 * lead factors, as the reference computes them with gamma_root (nested.rs:1036-1047) before its
 * solve: for instance i and block b (q = i * nblocks + b), w_left[q] is nl_b x left_channels[q] and
 * w_right[q] is nr_b x right_channels[q], column-major complex128, with W W^† = Γ = i(Σ - Σ^†) of
 * that block's lead at the slot's energy. Outputs, column-major complex128 with n rows (every
 * orbital of the system, region order): psi_left[i] has Σ_b left_channels[i * nblocks + b]
 * columns, block b's after those of the blocks before it and zero outside the block's orbitals
 * (the reference's concatenation, nested.rs:887-897); psi_right[i] likewise. status[i] per
 * instance (CAROLI_OK, CAROLI_REFINE_STALLED, CAROLI_NONFINITE ...).
 * Runs the mixed path: complex-f32 factors precondition an FP64 GMRES solve of A X = B with
 * B = [e_L W_L, e_R W_R], refined until the correction of the whole of X is below 1e-10 of X
 * (caroli_set_refine_options). */
int caroli_scattering_states(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots, const int32_t* configs,
                             const double* const* w_left, const int32_t* left_channels, const double* const* w_right,
                             const int32_t* right_channels, double* const* psi_left, double* const* psi_right,
                             int32_t* status);

/* Multi-terminal devices (NestedMultiTerminal, crates/caroli-green/src/nested_multi.rs): any number
 * of leads attached to the device, T_pq between every pair.
 * 1. caroli_plan_upload with, per block, the kept orbitals (every device orbital some lead couples
 *    to, the sites holding them excluded from `interior`) as its left list and an empty right list:
 *    the tree's root keeps them (nested_multi.rs:64-77, :297-303).
 * 2. caroli_multi_leads: `nleads` leads; the device orbitals of lead p in block b are
 *    lead_orbitals[lead_ptr[b * nleads + p] .. lead_ptr[b * nleads + p + 1]) (lead_ptr[0] = 0; an
 *    empty range for a lead the block does not reach), each one of the block's kept orbitals.
 * 3. caroli_multi_sigma_upload: Σ_p = V_p g_p V_p^† of every (block, lead) at one energy,
 *    sigma[b * nleads + p] column-major complex128 in the order of that lead's orbitals (NULL for an
 *    empty lead). The root subtracts their sum (nested_multi.rs:304-318).
 * 4. caroli_multi_transmissions: t[(i * nleads + p) * nleads + q] = T_pq = Tr[Γ_p G_pq Γ_q G_pq^†]
 *    from lead q into lead p, summed over the blocks (nested_multi.rs:337-364), for `count`
 *    instances (energy slot, configuration); CAROLI_DOUBLE or CAROLI_SINGLE, as the reference's
 *    Precision, or CAROLI_MIXED (no counterpart): X = A^-1 [W_1 ... W_P], W_p W_p^† = Γ_p, refined in
 *    FP64 from f32 factors and T_pq = Σ over lead q's columns of x(p)^† Γ_p x(p); block solves with
 *    more than 96 sources in all, or that the refinement cannot resolve, take the FP64 path.
 *    The two-terminal entry points refuse a plan with leads. */
int caroli_multi_leads(caroli_ctx* ctx, int plan_id, int nleads, const int64_t* lead_ptr, const int64_t* lead_orbitals);
/* Transmissions between sectors of the leads (NestedMultiTerminal::sector_transmissions,
 * nested_multi.rs:226-295): `nlabels` trace labels, label k on the orbitals of lead label_lead[k],
 * with its own broadening: gammas[(i * nblocks + b) * nlabels + k] (np x np column-major
 * complex128, in the order of that lead's orbitals in block b; NULL where the block has no part of
 * the lead) is Γ of the lead projected on the sector, V P_a i(g - g^†) P_a V^†. The root is the
 * one of the slot's self-energies (all leads whole). t[(i * nlabels + k) * nlabels + l] =
 * Tr[Γ_k G Γ_l G^†] from label l into label k, summed over blocks. CAROLI_DOUBLE or CAROLI_SINGLE. */
int caroli_multi_sector_transmissions(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots,
                                      const int32_t* configs, int precision, int nlabels, const int32_t* label_lead,
                                      const double* const* gammas, double* t, int32_t* status);
/* Scattering states of a multi-terminal device (NestedMultiTerminal::scattering_states,
 * nested_multi.rs:382-438): ψ_p = G W_p for every lead p. For instance i, block b and lead p
 * (q = (i * nblocks + b) * nleads + p), w[q] is np x channels[q] column-major complex128 with
 * W W^† = Γ_p on the lead's orbitals in the order of caroli_multi_leads (NULL for no channel).
 * psi[i * nleads + p] receives n x Σ_b channels columns, block b's after those of the blocks
 * before it, zero outside the block. Runs the mixed path (f32 factors, FP64 GMRES converged on the
 * whole of X), as caroli_scattering_states. */
int caroli_multi_scattering_states(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots,
                                   const int32_t* configs, const double* const* w, const int32_t* channels,
                                   double* const* psi, int32_t* status);
int caroli_multi_sigma_upload(caroli_ctx* ctx, int plan_id, int slot, double energy, const double* const* sigma);
int caroli_multi_transmissions(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots, const int32_t* configs,
                               int precision, double* t, int32_t* status);

/* The FP64 Green's function on the kept orbitals of every block's root (lead_green, nested.rs:783-802;
 * the root of NestedMultiTerminal::smatrix, nested_multi.rs:440-495): for instance i and block b
 * (q = i * nblocks + b), g[q] receives the kept x kept block of (z - H - Σ)^-1, column-major
 * complex128, kept[q] = its size. The kept orbitals are the left slice then the right one (or the
 * single list of a multi-terminal block), in the plan's order. The scattering matrix is formed
 * from it on the host. */
int caroli_root_green(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots, const int32_t* configs,
                      double* const* g, int32_t* kept, int32_t* status);

/* Transmission matrices t = W_L^† G_LR W_R of every block (transmission_eigenvalues and
 * fano_factor, nested.rs:753-780, take the squared singular values of t). For instance i and block
 * b (q = i * nblocks + b): w_left[q] is nl_b x left_channels[q] column-major complex128 with
 * W_L W_L^† = Γ_L; W_R is the slot's (caroli_sigma_upload). t[q] receives left_channels[q] x
 * right_channels[q] column-major complex128 (room for nr_b columns), right_channels[q] the slot's
 * channel count. Runs the mixed path: X = G W_R refined in FP64 (as the transmission), then
 * t = W_L^† X_L on the device. */
int caroli_transmission_matrix(caroli_ctx* ctx, int plan_id, int count, const int32_t* slots, const int32_t* configs,
                               const double* const* w_left, const int32_t* left_channels, double* const* t,
                               int32_t* right_channels, int32_t* status);

/* caroli_solve_batch over instances of several systems (plans) at once: instance i is
 * (plan_ids[i], slots[i], configs[i]), slots and configurations of that plan. Systems of different
 * sizes and trees (e.g. ribbons of many widths and lengths) share every level-synchronous launch.
 * The reference solves each system on its own (NestedTwoTerminal::transmission_with, nested.rs:682);
 * this batches a caller's loop over systems. */
int caroli_solve_multi(caroli_ctx* ctx, int count, const int32_t* plan_ids, const int32_t* slots,
                       const int32_t* configs, int precision, double* t, int32_t* status, double* err);

/* Device time of the last caroli_solve_batch (ms), and kernels it launched. */
int caroli_last_timing(const caroli_ctx* ctx, double* device_ms, int64_t* launches);

/* Of the last caroli_solve_batch: solves recomputed in double precision (CAROLI_MIXED points the
 * refinement could not resolve, as precision::checked recomputes failed points), and the largest
 * number of refinement iterations a solve took. */
int caroli_last_stats(const caroli_ctx* ctx, int64_t* fallbacks, int64_t* max_refine_iters);

/* Per block solve of the last caroli_solve_batch (as caroli_last_job_info): GMRES (Arnoldi) steps
 * of the mixed refinement, summed over its outer iterations (0 outside CAROLI_MIXED). */
int caroli_last_job_steps(const caroli_ctx* ctx, int64_t capacity, int32_t* steps, int64_t* count);
/* Per block solve of the last caroli_solve_batch (instance-major, blocks fastest; up to
 * `capacity` entries, *count = all): refinement iterations, pivots perturbed by static pivoting,
 * and status (100 + s: status s in reduced precision, then recomputed in double precision). */
int caroli_last_job_info(const caroli_ctx* ctx, int64_t capacity, int32_t* iters, int32_t* perturbed,
                         int32_t* status, int64_t* count);

/* Of the last caroli_solve_batch in CAROLI_MIXED: preconditioner applications (GMRES steps, one
 * forward and backward sweep each) summed over the block solves, and the steps the batch launched
 * (a step runs while any solve of the batch still iterates). No reference counterpart: the
 * reference has no iterative refinement. */
int caroli_last_refine_steps(const caroli_ctx* ctx, int64_t* job_steps, int64_t* batch_steps);

/* Refinement controls of CAROLI_MIXED (defaults 6, 1e-10, 1e-10): at most max_iters outer steps
 * (FP64 residual, GMRES on the f32 factors), done when the estimated relative error of the left
 * slice of the solution is at most tol; each GMRES runs until its residual falls by inner_tol.
 * No reference counterpart (precision::PrecisionOptions covers only the double recomputation). */
int caroli_set_refine_options(caroli_ctx* ctx, int max_iters, double tol, double inner_tol);

/* Rank-32 Schur updates of f32 fronts (CAROLI_MIXED, CAROLI_SINGLE) on the tcgen05 tensor cores
 * (3xTF32, default 1) or on the CUDA cores (0). No reference counterpart. */
int caroli_set_tensor_cores(caroli_ctx* ctx, int enable);

/* CAROLI_MIXED block solves whose sources (the right lead's open channels; every lead's for a
 * multi-terminal block) number more than `channels` take the FP64 path (default 96). No reference
 * counterpart. */
int caroli_set_mixed_max_channels(caroli_ctx* ctx, int channels);

/* Polls a pipeline wait of the tensor-core update may make before it gives up (default and
 * maximum 1 << 22; a negative value restores the default). A wait that runs out marks its solve
 * CAROLI_TIMEOUT (CAROLI_MIXED then recomputes it in FP64: status 105 in caroli_last_job_info)
 * after the copies and products already issued have drained; the context stays usable. Meant for
 * testing that path. No reference counterpart. */
int caroli_set_wait_limit(caroli_ctx* ctx, int64_t polls);

/* The autotuner (default on; no reference counterpart): the first time a set of plans is solved in
 * reduced precision, the f32 factorization of up to 256 of its block solves is timed under each
 * candidate schedule and the fastest is kept for that plan set and precision. Candidates: the
 * largest front factored by one CTA in shared memory (48, 64 or 96 variables; larger ones take
 * the panel sweep and rank-32 updates) x how those larger fronts are updated: (2) on the tensor
 * cores with the panels restricted to the pivot columns and the Schur complement [X; S] formed by
 * one GEMM per front, (1) on the tensor cores with rank-32 updates of every column, (0) on the CUDA
 * cores. A candidate replaces the default schedule (96, mode 1 when caroli_set_tensor_cores is on,
 * else 0) only when it is more than 5 % faster: the schedule also shapes the refinement, which the
 * trials do not time. Off: the default schedule. Changing it forgets the choices. */
int caroli_set_autotune(caroli_ctx* ctx, int enable);

/* The schedule used while the autotuner is off: small_max 48, 64 or 96 and the update mode 2, 1
 * or 0 as above (mode 1 or 2 also needs caroli_set_tensor_cores on). Default (96, 1). */
int caroli_set_schedule(caroli_ctx* ctx, int small_max, int update_mode);

/* Mixed-precision batches whose largest block solve carries at least `min_columns` right-hand-side
 * columns (channels) sweep their large fronts and roots as tensor-core GEMMs; others use the row
 * kernels. Default 32. No reference counterpart. */
int caroli_set_sweep_columns(caroli_ctx* ctx, int min_columns);

/* Threads of a CTA factoring a front of 64 to 96 variables in shared memory: 512 (default; twice
 * the warps replay the boundary rows) or 256. No reference counterpart. */
int caroli_set_small_threads(caroli_ctx* ctx, int threads);

/* CUDA graph replay (default on; no reference counterpart): a batch run twice in a row with the
 * same plans, schedule and device buffers has its factorization (every tree level's launches, the
 * root assembly and inverse) captured as a CUDA graph on its second run and replayed with one
 * launch afterwards. */
int caroli_set_graphs(caroli_ctx* ctx, int enable);

/* The schedule the last batch ran with: small_max, the update mode as above (tensor_cores = 2, 1
 * or 0), tuned = 1 when the autotuner chose them, trial_ms[9] (may be NULL) the trials'
 * factorization times in ms for small_max (48, 64, 96) x mode (2, 1, 0) (NaN: not tried), and the
 * factorization graphs replayed and captured so far. */
int caroli_last_schedule(const caroli_ctx* ctx, int32_t* small_max, int32_t* tensor_cores, int32_t* tuned,
                         double* trial_ms, int64_t* graph_replays, int64_t* graph_captures);

/* Device time of the last caroli_solve_batch split into the tree factorization, the root
 * inverse, and the rest (trace, or refinement and double-precision recomputations), in ms. */
int caroli_last_phases(const caroli_ctx* ctx, double* factor_ms, double* root_ms, double* tail_ms);

#ifdef __cplusplus
}
#endif
#endif /* CAROLI_GB300_H */

/*
 * jqmc_gpu.h -- C ABI of the GB300 (sm_103a) walker-path library libjqmc_gpu.so.
 *
 * All pointers named d_* are device pointers owned by the caller; host
 * descriptors are read during the call only.  Every entry point returns 0 on
 * success or a negative JQMC_E_* code; nothing throws across the ABI.  Calls
 * are asynchronous on the given CUDA stream (cudaStream_t passed as void*);
 * the library synchronises only inside jqmc_system_create/destroy and when a
 * mixed-form rebuild first grows the system's tensor-core workspace.
 *
 * Each entry point names the reference interface (jQMC, Python/JAX) whose
 * per-walker computation it replaces, batched over a leading walker axis.
 */
#ifndef JQMC_GPU_H
#define JQMC_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define JQMC_OK 0
#define JQMC_E_ARG (-1)       /* bad pointer / size / unsupported option     */
#define JQMC_E_LIMIT (-2)     /* size above a compiled maximum               */
#define JQMC_E_CUDA (-3)      /* a CUDA runtime call failed                  */
#define JQMC_E_SMEM (-4)      /* shared-memory footprint too large           */

#define JQMC_LMAX 6           /* highest AO angular momentum                 */
#define JQMC_ECP_SLOTS 8      /* channels per nucleus in the ECP table       */
#define JQMC_MAX_ELEC 256     /* N_up + N_dn                                 */
#define JQMC_MAX_NUP 128
#define JQMC_MAX_AO 4096
#define JQMC_MAX_ATOM 512
#define JQMC_ECACHE_STRIDE 24 /* doubles per electron in the energy cache    */

/* Walker status bits (per walker, OR-ed by the kernels). */
#define JQMC_ST_SINGULAR 1    /* zero pivot while inverting G                */
#define JQMC_ST_ZERO_RATIO 2  /* a chosen/accepted move had det ratio 0      */
#define JQMC_ST_NAN 4         /* non-finite weight or energy                 */

typedef struct jqmc_system jqmc_system; /* opaque: device copy of the tables */

/* One contracted-GTO basis.  shells: nshell rows of 8 int32
 *   {atom, l, nprim, prim0, ao0, nm, mfirst, kind}
 * kind 0, spherical: AO ao0+k of the shell carries m = mfirst+k, k < nm,
 * 1 <= nm <= 2l+1; prims: nprim rows of {Z, c*N_p*sqrt((2l+1)/4pi)} with N_p the
 * primitive normalisation of jqmc/atomic_orbital.py:2316-2323.
 * kind 1, Cartesian (jqmc/atomic_orbital.py:1984-2290): one AO (nm = 1),
 * x^nx y^ny z^nz with (nx, ny, nz) component mfirst of the shell's
 * (l+1)(l+2)/2 in TREXIO order; prims {Z, c*N_cart} with
 * N_cart = sqrt((2Z/pi)^(3/2) (8Z)^l nx!ny!nz!/((2nx)!(2ny)!(2nz)!)).
 * Shells are grouped by nucleus (atom non-decreasing). */
typedef struct {
  int32_t nshell, nao, nprim;
  const int32_t* shells;
  const double* prims;
} jqmc_basis_desc;

typedef struct {
  int32_t natom, n_up, n_dn;
  const double* atom_pos;        /* natom*3 (bohr)                           */
  const double* atom_zeff;       /* natom: Coulomb charges (Z - z_core)      */
  jqmc_basis_desc det;           /* geminal basis                            */
  const double* lambda;          /* det.nao^2, row-major, paired block in AOs*/
  int32_t has_j1, j1_type;       /* type 0 = exp, 1 = pade                   */
  double j1_param;
  const double* j1_zeff;         /* natom                                    */
  int32_t has_j2, j2_type;       /* type 0 = pade, 1 = exp                   */
  double j2_param;
  int32_t has_j3;
  jqmc_basis_desc j3;
  const double* j3_matrix;       /* j3.nao*(j3.nao+1), row-major; last column = j1 vector */
  int32_t ecp_flag;
  const int32_t* ecp_maxl1;      /* natom: index of the local channel        */
  const int32_t* ecp_chan;       /* natom*JQMC_ECP_SLOTS*2: (first term, count) per (atom, l) */
  int32_t ecp_nterm;
  const double* ecp_terms;       /* ecp_nterm*3: (c, n, alpha)               */
  int32_t nv;                    /* angular quadrature: 4, 6, 12 or 18       */
  const double* mesh_points;     /* nv*3 unit vectors                        */
  const double* mesh_weights;    /* nv                                       */
  double ion_ion;                /* constant ion-ion Coulomb energy          */
  int32_t nonlocal_move;         /* LRDMC non-local ECP moves (jqmc_gfmc.py:4941-5017):
                                  * JQMC_NONLOCAL_TMOVE or JQMC_NONLOCAL_DLTMOVE */
} jqmc_system_desc;

/* Non-local ECP moves of the LRDMC projections and energies.  T-move: the
 * element V = w_q V_l P_l psi(r')/psi(r); dltmove (determinant locality):
 * V_det with the determinant ratio alone, SP part max(V_det, 0), move weight
 * min(V_det, 0) times the Jastrow ratio.  The VMC energy always uses psi. */
#define JQMC_NONLOCAL_TMOVE 0
#define JQMC_NONLOCAL_DLTMOVE 1

/* Walker-table precision. */
#define JQMC_PREC_FP64 0      /* every table and every operation in double       */
#define JQMC_PREC_MIXED 1     /* G, G^-1, T_up, T_dn, h3 float; AO values, ratios  */
                              /* and rank-1 updates float; AO gradients/Laplacians,*/
                              /* energy cache, weights and the table rebuild double;*/
                              /* block energy (jqmc_lrdmc_energy): float values     */
                              /* with compensated float-float sums over the FP64-   */
                              /* accurate tables (jqmc_walkers.tlo); the walkers    */
                              /* whose mesh ratios cancel strongly (factor above    */
                              /* JQMC_FAST_ENERGY_CANCEL) recomputed in FP64        */
#define JQMC_PREC_MIXED_FASTE 2 /* as JQMC_PREC_MIXED, the compensated energy alone */
                                /* (rare configurations with errors of 1e-4 Ha)     */
/* Cancellation factor above which a walker's block energy is recomputed in FP64:
 * C = sum_i |w_i| M_i / sum_i |w_i ratio_i| over the walker's mesh elements
 * (weight w_i, ratio psi(r')/psi(r) = sum_a phi_a(r') T_a times the Jastrow
 * factor, M_i the same sum over |phi_a T_a|).  On the 32-nucleus chain's
 * sampled configurations fewer than 0.1 % exceed 10.  After jqmc_lrdmc_energy
 * in JQMC_PREC_MIXED, C is the first double of each walker's scratch block. */
#define JQMC_FAST_ENERGY_CANCEL 10.0

/* Per-walker state, all device arrays (N = n_up + n_dn, n = n_up, A = det.nao,
 * A3 = j3.nao).  Electron-major layouts: electron e's vectors are contiguous.
 * Table element type: double for JQMC_PREC_FP64, float for JQMC_PREC_MIXED. */
typedef struct {
  int32_t nwalk;
  int32_t precision;  /* JQMC_PREC_*                                             */
  double* r;          /* nwalk*N*3, up electrons first (always double)           */
  void* G;            /* nwalk*n*n geminal matrix                                */
  void* Ginv;         /* nwalk*n*n                                               */
  void* Tup;          /* nwalk*n*A: row i = lambda Phi_dn G^-1 [:, i]            */
  void* Tdn;          /* nwalk*n*A: row j = (G^-1 Phi_up^T lambda)[j, :]         */
  void* h3;           /* nwalk*N*A3 J3 field: dJ3/dphi3(r_e) (unused if no J3)   */
  void* dphi;         /* nwalk*N*4*A: grad x, y, z and Laplacian of every geminal */
                      /* AO at each electron (kept current by every move)       */
  void* dphi3;        /* nwalk*N*5*A3: value, grad x, y, z, Laplacian of the J3  */
                      /* AOs at each electron (unused if no J3)                  */
  double* ecache;     /* nwalk*(N+1)*JQMC_ECACHE_STRIDE: per-electron e-ion and  */
                      /* local-ECP energies, J1/J2 grad/lap, nearest nucleus and */
                      /* non-local channel values; last row: e-e Coulomb total   */
  double* scratch;    /* JQMC_PREC_MIXED: nwalk*2*n*A doubles used by the FP64   */
                      /* rebuilds (jqmc_walker_init, jqmc_lu_rebuild_refine);    */
                      /* unused for JQMC_PREC_FP64                               */
  float* dcache;      /* JQMC_PREC_MIXED: nwalk*N*(natom+N)*3 floats of electron */
                      /* displacements, required when that exceeds 64 KiB per    */
                      /* walker (else kept in shared memory); may be NULL below  */
  int32_t* status;    /* nwalk JQMC_ST_* bits                                    */
  float* tlo;         /* JQMC_PREC_MIXED, optional: per walker 2*n*A + N*A3      */
                      /* floats, the low parts of the FP64-accurate T tables     */
                      /* (T_up rows, then T_dn rows) followed by those of the J3 */
                      /* field (N rows of A3; A3 = 0 without J3): written by     */
                      /* jqmc_walker_init and jqmc_lu_rebuild_refine when        */
                      /* non-NULL; read by jqmc_lrdmc_energy when non-NULL,      */
                      /* which the caller may pass only while no move has        */
                      /* changed the tables since that build.  With it the block */
                      /* energy is computed from T_hi + T_lo, h_hi + h_lo and AO */
                      /* values, gradients and Laplacians re-evaluated in FP64   */
                      /* at the electrons instead of the float tables, and the   */
                      /* non-local ECP ratios of the electrons whose elements    */
                      /* weigh most are recomputed in FP64.                      */
} jqmc_walkers;

/* Copy the tables to the current device.  Replaces the per-call packing of
 * AOs_sphe_data / Geminal_data / Jastrow_data / Coulomb_potential_data
 * (jqmc/atomic_orbital.py:781-929, determinant.py:94-141,
 * jastrow_factor.py:561-1476, coulomb_potential.py:188-598). */
int jqmc_system_create(const jqmc_system_desc* desc, jqmc_system** out);
int jqmc_system_destroy(jqmc_system* sys);

/* 1 when the mixed form's table rebuild (jqmc_walker_init, jqmc_lu_rebuild_refine)
 * forms M = Phi lambda on the tensor cores (tcgen05, split-bf16 operands with
 * exact FP32 sums, about 1e-12 of sum |Phi| |lambda|) -- systems with at most
 * 768 geminal AOs -- and 0 when it uses the float-float CUDA-core kernel.  The tensor-core
 * path keeps an operand workspace with the system (about 12 bytes per
 * electron-row x AO for up to 65536 rows, allocated on the first rebuild); a
 * rebuild that would have to allocate it inside a stream capture uses the
 * CUDA-core kernel instead.  Rebuilds of one system must not overlap on
 * different streams (they share the workspace).  Replaces the geminal assembly
 * lambda . Phi of jqmc/determinant.py:1380-1402 in the rebuild. */
int32_t jqmc_tensor_core_rebuild(const jqmc_system* sys);

/* Bytes of walker state per walker (sum over the jqmc_walkers arrays) for a
 * JQMC_PREC_* precision. */
int64_t jqmc_walker_bytes(const jqmc_system* sys, int32_t precision);

/* AO values, gradients and Laplacians at npts points of basis 0 (geminal) or
 * 1 (J3).  d_out: 5*nao*npts = (val, gx, gy, gz, lap), AO-major.
 * Replaces compute_AOs_value_grad_lap (jqmc/atomic_orbital.py:3594-3640) and,
 * through its first block, compute_AOs (atomic_orbital.py:1886). */
int jqmc_ao_vgl(const jqmc_system* sys, int32_t basis, const double* d_r, int64_t npts, double* d_out, void* stream);

/* Build every walker's state from its positions w->r: AO tables, G (geminal,
 * jqmc/determinant.py:1380-1402), G^-1 by LU with partial pivoting (in place
 * of the SVD pseudo-inverse of jqmc_mcmc.py:4249-4261 / jqmc_gfmc.py:691),
 * T tables and the J3 field. */
int jqmc_walker_init(const jqmc_system* sys, const jqmc_walkers* w, void* stream);

/* Rebuild the tables that Sherman-Morrison updates carry -- G, G^-1 (LU with
 * partial pivoting plus one FP64 refinement step X <- X + X(I - G X)), the T
 * tables and the J3 field -- from the positions, in FP64, and store them in the
 * walkers' table type.  The energy cache and the AO derivative tables are left
 * as they are (every move recomputes them exactly).  Replaces the per-branching
 * inverse recomputation of GFMC_n (jqmc/jqmc_gfmc.py:4706-4717, :6319) and is
 * the periodic FP64 rebuild of the mixed-precision form. */
int jqmc_lu_rebuild_refine(const jqmc_system* sys, const jqmc_walkers* w, void* stream);

/* ln|det G| and its sign per walker from G (LU, jqmc/determinant.py:1026-1111),
 * plus the Jastrow value J (jastrow_factor.py:2127-2178).  JQMC_PREC_FP64 only. */
int jqmc_log_psi(const jqmc_system* sys, const jqmc_walkers* w, double* d_logdet, double* d_sign, double* d_jastrow, void* stream);

/* Per-electron derivatives of ln|psi| and kinetic elements, FP64 walkers:
 * d_out (nwalk, N, 9) = (grad ln|det| (3), lap ln|det|, grad J (3), lap J,
 * T_e = -1/2 (lap ln psi + |grad ln psi|^2)) for every electron, up spin first.
 * Replaces compute_grads_and_laplacian_ln_Det (jqmc/determinant.py:1809),
 * compute_grads_and_laplacian_Jastrow_part (jqmc/jastrow_factor.py:2983) and
 * compute_kinetic_energy_all_elements (jqmc/wavefunction.py:1081). */
int jqmc_electron_terms(const jqmc_system* sys, const jqmc_walkers* w, double* d_out, void* stream);

/* Discretised kinetic elements, FP64 walkers: d_el (nwalk, N, 6) =
 * -psi(r_e + alat s_k)/psi(r) / (2 alat^2) for every electron e (up spin
 * first) and the moves s_k = +x, -x, +y, -y, +z, -z of the rotation
 * R(d_angles[w]) (Euler angles as in jqmc_vmc_measure), i.e. the rows of
 * R^T.  Replaces compute_discretized_kinetic_energy (jqmc/wavefunction.py:1620). */
int jqmc_kinetic_mesh(const jqmc_system* sys, const jqmc_walkers* w, const double* d_angles, double alat, double* d_el,
                      void* stream);

/* Per-walker derivatives of ln|psi| with respect to the variational parameters,
 * FP64 walkers only, from the positions and G^-1 (AO values are recomputed, not
 * stored).  Replaces the per-walker grad(evaluate_ln_wavefunction) of
 * jqmc_mcmc.py:856-876 with the blocks of collect_param_grads
 * (jastrow_factor.py:2110-2124, determinant.py:389-399):
 *   d_j1     nwalk           d ln psi / d jastrow_1b_param
 *   d_j2     nwalk           d ln psi / d jastrow_2b_param
 *   d_j3     nwalk*A3*(A3+1) d ln psi / d j_matrix (last column: one-body vector)
 *   d_lambda nwalk*A*A       d ln psi / d lambda in the AO basis of the tables
 *                            (a caller holding MO-basis lambda maps it with the
 *                            MO coefficients: C_up D C_dn^T)
 * d_work: nwalk*2*n*A doubles, required with d_lambda.  A NULL output skips its
 * block; 0 is written for an absent J1 / J2 term. */
int jqmc_dlnpsi_dparam(const jqmc_system* sys, const jqmc_walkers* w, double* d_j1, double* d_j2, double* d_j3,
                       double* d_lambda, double* d_work, void* stream);

/* d ln|psi| / dR for every nucleus (FP64 walkers, current positions and cached
 * tables): the Pulay term force_PP of jqmc_mcmc.py:780-845 (dln_Psi/dR without
 * space warp), which the reference obtains as grad(evaluate_ln_wavefunction)
 * with respect to the nuclear positions (jqmc_mcmc.py:782-793).
 * d_out: nwalk*natom*3. */
int jqmc_dlnpsi_dR(const jqmc_system* sys, const jqmc_walkers* w, double* d_out, void* stream);

/* K Metropolis proposals per walker (jqmc_mcmc.py:4316-4523, fori_loop body),
 * explicit draws: d_idraw nwalk*K*4 int32 (sel in [0,N), up index, dn index,
 * axis), d_fdraw nwalk*K*2 double (standard normal, uniform).  Adds the number
 * of accepted moves to d_accept[w].  JQMC_PREC_FP64 only. */
int jqmc_vmc_sweep(const jqmc_system* sys, const jqmc_walkers* w, int32_t K, const int32_t* d_idraw,
                   const double* d_fdraw, double Dt, double eps_AS, int32_t* d_accept, void* stream);

/* Local energy and AS weight per walker (jqmc/hamiltonians.py:225-290 with the
 * non-local ECP on the rotated quadrature, coulomb_potential.py:1478-1712;
 * w_L = (R_AS / max(R_AS, eps))^2, jqmc_mcmc.py:743-747).  d_angles: nwalk*3
 * Euler angles; the rotation is R(angles) of jqmc_mcmc.py:4228-4245.
 * JQMC_PREC_FP64 only. */
int jqmc_vmc_measure(const jqmc_system* sys, const jqmc_walkers* w, const double* d_angles, double eps_AS,
                     double* d_eL, double* d_wL, void* stream);

/* K LRDMC fixed-count projections per walker (GFMC_n, jqmc_gfmc.py:4779-5166),
 * T-move ECP treatment.  d_draw nwalk*K*4 = (alpha, beta, gamma, u_move).
 * d_w is multiplied by the K step weights b_x.  Both precisions. */
int jqmc_lrdmc_project(const jqmc_system* sys, const jqmc_walkers* w, int32_t K, const double* d_draw, double alat,
                       double E_scf, double* d_w, void* stream);

/* e_L = V_diag + V_nondiag and V_diag at the current positions with the
 * rotation of d_draw (nwalk*4, the last step's draw): jqmc_gfmc.py:5361-5640. */
int jqmc_lrdmc_energy(const jqmc_system* sys, const jqmc_walkers* w, const double* d_draw, double alat,
                      double* d_eL, double* d_vdiag, void* stream);

/* Continuous-time LRDMC projections (GFMC_t, jqmc_gfmc.py:724-1107 and the
 * while loop :1539-1620).  Each walker projects until its remaining time
 * d_tau_left (in/out) is spent or its K draws are used: per step
 * d_draw[w][k] = (alpha, beta, gamma, xi, u_move) (nwalk*K*5),
 * tau_update = min(tau_left, ln(1 - xi) / V_nondiag), d_w *= exp(-tau_update e_L),
 * and the move is made only while time is left.  d_nsteps (out): projections
 * made by this call; d_eL (out): e_L of the step that spent the time (left
 * unchanged for a walker whose draws ran out first -- call again with new
 * draws).  Both precisions. */
int jqmc_lrdmc_project_t(const jqmc_system* sys, const jqmc_walkers* w, int32_t K, const double* d_draw, double alat,
                         double* d_w, double* d_tau_left, int32_t* d_nsteps, double* d_eL, void* stream);

/* Stochastic reconfiguration with one comb draw zeta (jqmc_gfmc.py:2010-2090):
 * d_chosen[k] = first j with cumsum(w/sum w)[j] >= (k + zeta)/nwalk (clamped
 * to nwalk-1).  d_cum: caller-provided scratch of nwalk doubles that receives
 * the cumulative normalised weights. */
int jqmc_branch_comb(int32_t nwalk, const double* d_w, double zeta, int32_t* d_chosen, double* d_cum, void* stream);

/* dst walker k <- src walker d_chosen[k] for every state array (walker
 * migration of jqmc_gfmc.py:2100-2266 on one device). */
int jqmc_walker_gather(const jqmc_system* sys, const jqmc_walkers* src, const jqmc_walkers* dst,
                       const int32_t* d_chosen, void* stream);

/* Allocation-free form of jqmc_branch_comb.  It has no counterpart in the
 * reference.  It is for callers that cannot allocate device memory -- for
 * example a host code whose own pool has reserved the GPU's memory, or a
 * driver loop that must not wait on an allocation -- so they need not find a
 * scratch buffer: the cumulative weights go to a fixed device array of
 * JQMC_NOALLOC_MAX_WALKERS doubles (2 MiB) that the library holds on every GPU
 * that loads it until the process exits.  nwalk above that limit returns
 * JQMC_E_LIMIT; no cudaMalloc/cudaFree is called.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) with that device
 * current; make that first call before any stream capture.  The look-up is
 * repeated on the first call after the device's context was replaced (e.g. by
 * cudaDeviceReset), which reloads the array.  All calls share
 * the one array, so calls that overlap on the GPU (other streams, other host
 * threads) race: serialise them. */
#define JQMC_NOALLOC_MAX_WALKERS 262144
int jqmc_branch_comb_noalloc(int32_t nwalk, const double* d_w, double zeta, int32_t* d_chosen, void* stream);

/* Measurement helper (no reference counterpart): launches a kernel of
 * 8 independent FP64 FMA chains per thread (blocks x 256 threads, iters
 * iterations) and returns in *flops the FP64 operations it performs, so that a
 * caller timing it obtains the device's FP64 FMA throughput. */
int jqmc_probe_fp64(int64_t iters, int32_t blocks, double* d_sink, double* flops, void* stream);

/* The same for FP32 FMA chains (measurement helper, no reference counterpart). */
int jqmc_probe_fp32(int64_t iters, int32_t blocks, float* d_sink, double* flops, void* stream);

/* ---- Batches of systems (many molecules in one launch) --------------------
 * A batch binds N (system, walker set) pairs of one precision; the walkers of
 * item i are walkers [off_i, off_i + nwalk_i) of the batch, off_i the running
 * sum of the earlier items' walker counts.  One launch covers every walker of
 * every item (each CTA finds its item), so molecules of uneven size share the
 * GPU; the per-item kernel parameters live on the device, so the launches can
 * be captured in a CUDA graph.  Replaces the per-molecule VMC driver loop of
 * jqmc_mcmc.py (MCMC.run, :456-1000) for many independent molecules. */
typedef struct jqmc_batch jqmc_batch;
int jqmc_batch_create(int32_t nitem, const jqmc_system* const* systems, const jqmc_walkers* walkers, jqmc_batch** out);
int jqmc_batch_destroy(jqmc_batch* b);
int jqmc_batch_walkers(const jqmc_batch* b);   /* total walkers of the batch */

/* K Metropolis proposals for every walker of the batch (the jqmc_vmc_sweep
 * step, jqmc_mcmc.py:4316-4523): d_idraw total*K*4 and d_fdraw total*K*2 in
 * batch walker order, d_accept total.  JQMC_PREC_MIXED batches run the
 * proposals with float tables (AO values, ratio, candidate G^-1 for the AS
 * factor, rank-1 updates) and double acceptance.  threads: CTA size (32..256,
 * a multiple of 32).  caches == 0 skips keeping the AO derivative tables and
 * the energy cache current (call jqmc_batch_rebuild with full = 1 before an
 * energy is measured). */
int jqmc_vmc_sweep_batch(const jqmc_batch* b, int32_t K, const int32_t* d_idraw, const double* d_fdraw, double Dt,
                         double eps_AS, int32_t* d_accept, int32_t threads, int32_t caches, void* stream);

/* full == 0: the drift-control rebuild of jqmc_lu_rebuild_refine for every
 * walker of the batch (JQMC_PREC_MIXED: the J3 field computed in float, as it
 * is stored); full != 0: jqmc_walker_init (all state in FP64, including the
 * energy cache and derivative tables; call it before an energy is measured). */
int jqmc_batch_rebuild(const jqmc_batch* b, int32_t full, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* JQMC_GPU_H */

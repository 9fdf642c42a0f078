/* quiqbox_gb300.h — C ABI of the GB300 (sm_103a) integral and Hartree–Fock path.
 *
 * Drop-in native back end for Quiqbox.jl's Gaussian-orbital integral API and
 * its RHF/UHF driver.  Plain C types only: the Julia side (basis containers,
 * parameter graph, SCF configuration) stays in Julia and binds these symbols
 * with `ccall`.  All matrices are column-major (Julia's layout).
 *
 * Conventions
 *  - A basis is `nfun` contracted functions; function f owns the primitives
 *    fun_ptr[f] .. fun_ptr[f+1]-1.  Every primitive has its own centre, Cartesian
 *    powers (i,j,k), exponent and *effective* weight: the contraction coefficient
 *    with every normalisation factor already applied, exactly the weights that
 *    `getOrbCorePointers` / `buildOrbCoreWeight!` produce
 *    (src/Integration/Framework.jl:748-825).
 *  - Outputs are caller-allocated host arrays; the library owns all device memory
 *    and keeps no pointer to caller memory after a call returns.
 *  - Every entry point returns a status (QB_OK or QB_ERR_*) and never aborts;
 *    qb_last_error() gives the message.  One context must not be used by two
 *    threads at once.
 */
#ifndef QUIQBOX_GB300_H
#define QUIQBOX_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    QB_OK = 0,
    QB_ERR_ARG = 1,            /* bad pointer / argument  (AssertionError, src/Exception.jl)          */
    QB_ERR_DIM = 2,            /* size mismatch           (DimensionMismatch, src/HartreeFock.jl:200) */
    QB_ERR_DOMAIN = 3,         /* out-of-domain value     (DomainError, src/HartreeFock.jl:989,994)   */
    QB_ERR_CUDA = 4,           /* CUDA runtime failure                                                */
    QB_ERR_TIMEOUT = 5,        /* a bounded device wait ran out                                       */
    QB_ERR_NOT_CONVERGED = 6,  /* SCF stopped without convergence (converged = false, :800)           */
    QB_ERR_NOMEM = 7,          /* device allocation failed                                            */
    QB_ERR_UNSUPPORTED = 8     /* angular momentum beyond the kernels' limits                         */
};

typedef struct qb_ctx qb_ctx;

typedef struct {
    int nfun;
    const int* fun_ptr;     /* nfun + 1                   */
    const double* center;   /* 3 * nprim, (x, y, z) each  */
    const int* ijk;         /* 3 * nprim                  */
    const double* alpha;    /* nprim                      */
    const double* weight;   /* nprim, effective weights   */
} qb_basis;

/* Context: one per host thread; owns device buffers, streams and the Boys table. */
int qb_create(qb_ctx** out, int device);
void qb_destroy(qb_ctx* ctx);
const char* qb_last_error(const qb_ctx* ctx);
int qb_device_info(qb_ctx* ctx, int* sm_count, int* cc_major, int* cc_minor);

/* One-electron matrices, nfun x nfun.
 * overlaps        <- src/Integration/Interface.jl:46  (overlaps)
 * elecKinetics    <- src/Integration/Interface.jl:143 (elecKinetics)
 * nucAttractions  <- src/Integration/Interface.jl:236 (nucAttractions; V = -sum_C Z_C (a|1/r_C|b))
 * coreHamiltonian <- src/Integration/Interface.jl:288 (coreHamiltonian = kinetic + nuclear) */
int qb_overlaps(qb_ctx* ctx, const qb_basis* basis, double* S);
int qb_elec_kinetics(qb_ctx* ctx, const qb_basis* basis, double* T);
int qb_nuc_attractions(qb_ctx* ctx, const qb_basis* basis, int nnuc, const double* Z, const double* R,
                       double* V);
int qb_core_hamiltonian(qb_ctx* ctx, const qb_basis* basis, int nnuc, const double* Z, const double* R,
                        double* H);

/* Multipole moments M_ij = <i| (x-Cx)^nx (y-Cy)^ny (z-Cz)^nz |j>, nfun x nfun, column-major.
 * Replaces multipoleMoments (src/Integration/Interface.jl:95; sampler Samplers.jl:19-21,
 * primitive integrals GaussianOrbitals.jl:184-247).  degrees[k] >= 0; per axis the left
 * and right Cartesian powers plus degrees[k] may not exceed 26 (QB_ERR_UNSUPPORTED). */
int qb_multipole_moments(qb_ctx* ctx, const qb_basis* basis, const double center[3], const int degrees[3],
                         double* M);

/* Autotuner of the direct J/K build (no counterpart in the reference): on the basis of the
 * last qb_jk_prepare and the uploaded density, times every compiled kernel variant of
 * every angular-momentum class on its actual quartet work list (best of `repeats`) and
 * keeps the fastest per class for this context; variants[c] (nclass entries of
 * qb_jk_stats, may be NULL) receives the choice (0: one quartet per thread, 1-4: warp-
 * cooperative configurations, 5: segmented kernel).  Costs a few J/K builds; J and K stay
 * those of the density. */
int qb_jk_autotune(qb_ctx* ctx, int repeats, int* variants);

/* Per-class device time of the J/K build (no counterpart in the reference, a measurement
 * hook): after qb_jk_prepare and a density upload, launches every class kernel alone with
 * its current variant over its work list on the context stream and times it with CUDA
 * events, best of `repeats`; ms[c] (nclass entries of qb_jk_stats) receives the time, 0 for
 * classes without work.  J and K stay those of the density. */
int qb_jk_class_times(qb_ctx* ctx, int repeats, float* ms);

/* Kernels of the learned initial guess (no counterpart in the reference): a small MLP
 * with BF16 weights and activations and FP32 accumulation, trained and evaluated on the
 * GPU (quiqbox.jl_gb300/guess.py builds the passes from these).  Device pointers; stream
 * is a cudaStream_t.  Matrices are row-major.
 * qb_bf16_gemm_nt: C (M x N, fp32) = A (M x K, bf16) * B^T (B: N x K, bf16) [+ bias (N)],
 *   tensor cores (mma.sync BF16 -> FP32); M and N multiples of 64, K of 32, A and B
 *   16-byte aligned.
 * qb_gelu_forward: a (bf16) = GELU(z); qb_gelu_backward: dz = da * GELU'(z).
 * qb_f32_to_bf16: y = bf16(x) (rows x cols) or its transpose (transpose != 0).
 * qb_bf16_transpose: y (cols x rows) = x^T.
 * qb_colsum: out[j] = sum_i x[i][j] (bias gradients).
 * qb_mse_grad: dy = 2 w (y - t) / wsum and *loss += sum w (y - t)^2 / wsum.
 * qb_adam_step: Adam (bias-corrected, step >= 1) on FP32 weights w with moments m, v;
 *   refreshes the BF16 copy w_bf16 when non-NULL. */
int qb_bf16_gemm_nt(int M, int N, int K, const void* A, const void* B, const float* bias, float* C, void* stream);
int qb_gelu_forward(int64_t n, const float* z, void* a, void* stream);
int qb_gelu_backward(int64_t n, const float* z, const float* da, float* dz, void* stream);
int qb_f32_to_bf16(int rows, int cols, const float* x, void* y, int transpose, void* stream);
int qb_bf16_transpose(int rows, int cols, const void* x, void* y, void* stream);
int qb_colsum(int rows, int cols, const float* x, float* out, void* stream);
int qb_mse_grad(int64_t n, const float* y, const float* t, const float* w, float wsum, float* dy, float* loss,
                void* stream);
int qb_adam_step(int64_t n, float* w, const float* g, float* m, float* v, void* w_bf16, float lr, float b1, float b2,
                 float eps, int step, void* stream);

/* Learned guess inputs and outputs on the device (one thread per atom pair (a, b), a <= b,
 * global atom indices; molecule m owns atoms [mol_atom0[m], mol_atom0[m] + mol_natom[m]);
 * atom_el: 0 H, 1 C, 2 N, 3 O; minimal basis, functions 1s (H) or 1s 2s 2px 2py 2pz).
 * qb_guess_features: X (npair x 128 fp32, row-major) = the pair's network input, R
 *   (npair x 9, row-major 3 x 3) = its local frame (columns: local x, y, z axes).
 * qb_guess_assemble: per-spin densities D (column-major, molecule m at D + mol_off[m],
 *   mol_n[m] x mol_n[m]) from the network's local-frame 5 x 5 blocks Y (row p, leading
 *   dimension ldy >= 25): block (a, b) = T Y_p T^T with T = diag(1, 1, R_p), written to
 *   the (a, b) and (b, a) blocks; atom_f0 = first function of each atom in its molecule. */
int qb_guess_features(int npair, const int* pair_mol, const int* pair_a, const int* pair_b, const int* mol_atom0,
                      const int* mol_natom, const double* atom_pos, const int* atom_el, const float* mol_charge,
                      float* X, double* R, void* stream);
int qb_guess_assemble(int npair, const int* pair_mol, const int* pair_a, const int* pair_b, const int* atom_el,
                      const int* atom_f0, const long long* mol_off, const int* mol_n, const float* Y, int ldy,
                      const double* R, double* D, void* stream);

/* Backward pass of the two-electron energy for basis-parameter gradients (the reference
 * has no analytic gradient; src/Differentiation/Finite.jl holds finite-difference
 * weights only).  Functions [0, n) of `basis` are the basis, [n, nfun) extra single
 * primitives g (derivative primitives); P is the n x n total density.  Recomputes every
 * (g nu|lambda sigma) (no storage) and returns, row-major ng x n,
 *   Jx[g][nu] = sum (g nu|lambda sigma) P_{lambda sigma},
 *   Kx[g][lambda] = sum (g nu|lambda sigma) P_{nu sigma}. */
int qb_adjoint_jk(qb_ctx* ctx, const qb_basis* basis, int n, const double* P, double* Jx, double* Kx);

/* k lowest eigenpairs of a symmetric n x n matrix A (column-major), n <= 1024: the
 * batched SCF's eigensolver (Householder tridiagonalisation, bisection, inverse
 * iteration).  w: k eigenvalues ascending; Y: n x k eigenvectors (column-major).  It
 * replaces the eigen call of solveFockMatrix (src/HartreeFock.jl:46-56) where only the
 * occupied orbitals are needed. */
int qb_eigh_lowest(qb_ctx* ctx, int n, int k, const double* A, double* w, double* Y);

/* Boys function sequence on the device: F[i*(M+1) + m] = F_m(T[i]), m = 0..M, T[i] >= 0.
 * Replaces computeBoysSequence (src/Integration/Engines/BoysFunction.jl:67-77) and
 * computeBoysFunc (:62-64).  path 0: the evaluator of the ERI class kernels (M <= 8);
 * path 1: the evaluator of the generic kernels (M <= 32). */
int qb_boys(qb_ctx* ctx, int n, const double* T, int M, int path, double* F);

/* Two-electron integrals (chemists' notation (ij|kl)).
 * qb_elec_repulsions <- src/Integration/Interface.jl:356 (elecRepulsions): nfun^4 tensor [i,j,k,l]
 * qb_elec_repulsion_list <- src/Integration/Interface.jl:331 (elecRepulsion) for nq explicit
 *                           0-based quartets (4 ints each) */
int qb_elec_repulsions(qb_ctx* ctx, const qb_basis* basis, double* eri);
int qb_elec_repulsion_list(qb_ctx* ctx, const qb_basis* basis, int64_t nq, const int* quartets,
                           double* out);

/* Direct Coulomb and exchange matrices of a symmetric density D, no stored ERIs:
 *   J_ij = sum_kl (ij|kl) D_kl,   K_ij = sum_kl (ik|jl) D_kl.
 * Replaces the stored-tensor contraction of getGcore (src/HartreeFock.jl:305-319):
 * G = 2J(D) - K(D) for RHF, G^s = J(Da+Db) - K(D^s) for UHF.
 * Shell quartets with Q_ab Q_cd max|D| < schwarz are skipped (Q = Schwarz factors). */
int qb_jk(qb_ctx* ctx, const qb_basis* basis, const double* D, double schwarz, double* J, double* K);

/* Split form of qb_jk for callers that keep the density on the device between
 * builds (and for timing): prepare the basis once, then upload / execute / download. */
int qb_jk_prepare(qb_ctx* ctx, const qb_basis* basis, double schwarz);
int qb_jk_upload_density(qb_ctx* ctx, const double* D);
int qb_jk_execute(qb_ctx* ctx);
int qb_jk_download(qb_ctx* ctx, double* J, double* K);

typedef struct {
    int shell_path;               /* 1: generated shell-class kernels, 0: generic per-function kernels */
    int nshell, npair, nclass;
    int64_t quartets;             /* canonical shell quartets surviving the screening (last execute)  */
    int64_t prim_quartets;        /* primitive quartets evaluated (last execute)                      */
    double flops;                 /* FP64 flops of the last execute (generated-code op counts)        */
    double ms_last;               /* device time of the last execute (CUDA events)                    */
    int64_t class_quartets[32];
    int64_t class_prim_quartets[32];
    int class_l[32][4];
} qb_jk_stats;
int qb_jk_get_stats(qb_ctx* ctx, qb_jk_stats* stats);

/* Introspection (no reference counterpart): the shell-pair table of the prepared
 * basis in the order the J/K kernels use it, grouped by pair class (la, lb) and
 * sorted by descending Schwarz factor within a class.  Pass null arrays to get
 * *npair only; otherwise each array holds *npair entries.  fa / fb are the first
 * function indices of the two shells (A is the shell of higher angular momentum). */
int qb_jk_pair_table(qb_ctx* ctx, int* npair, int* fa, int* fb, int* la, int* lb, double* Q);

/* J and K restricted to an explicit list of shell quartets (a test hook for the class
 * kernels, no reference counterpart): the sum over the listed quartets of the terms the
 * full build (qb_jk_execute, replacing getGcore, src/HartreeFock.jl:305-319) adds for them,
 * with the density of the last qb_jk_upload_density and each class's current kernel
 * variant.  pairs holds 2 * nq indices into the pair table of qb_jk_pair_table: bra pair,
 * ket pair, in canonical order (the ket's pair class not above the bra's; within one class
 * the ket index not above the bra index), else QB_ERR_ARG.  No Schwarz screening is
 * applied to the listed quartets; the kernels' primitive screening is. */
int qb_jk_quartet_list(qb_ctx* ctx, int64_t nq, const int* pairs, double* J, double* K);

/* Hartree–Fock SCF (runHartreeFock, src/HartreeFock.jl:953-1228) on the GPU:
 * symmetric orthogonalisation, Jacobi diagonalisation, direct J/K Fock build,
 * DD / DIIS / EDIIS / ADIIS convergence methods with the reference's three DIIS
 * coefficient solvers (constraintSolver!, src/HartreeFock.jl:1479-1487):
 * QB_DIIS_LBFGS (L-BFGS-B, the default :17), QB_DIIS_SPGB (spectral projected
 * gradient) and QB_DIIS_LCM (Lagrange multipliers, CMsolver!). */
enum { QB_SCF_DD = 0, QB_SCF_DIIS = 1, QB_SCF_EDIIS = 2, QB_SCF_ADIIS = 3 };
enum { QB_DIIS_LBFGS = 0, QB_DIIS_SPGB = 1, QB_DIIS_LCM = 2 };
enum { QB_GUESS_COREH = 0, QB_GUESS_GWH = 1, QB_GUESS_SAD = 2, QB_GUESS_DIRECT = 3 };

typedef struct {
    int uhf;                      /* 0 RHF (n_alpha == n_beta required), 1 UHF                   */
    int guess;                    /* QB_GUESS_*                                                  */
    const double* C0;             /* QB_GUESS_DIRECT: (1 or 2) nfun x nfun coefficient matrices */
    int nmethod;                  /* 1..8                                                        */
    int method[8];                /* QB_SCF_*                                                    */
    double interval[8];           /* per-method stopping thresholds; the last converges          */
    double secondary_ratio[2];    /* RMS(FDS-SDF) and RMS(dD) ratios (default 1000, 1000)        */
    double oscillate_threshold;   /* default 5e-6                                                */
    int max_step;                 /* default 200                                                 */
    int early_stop;               /* default 1                                                   */
    int diis_size;                /* default 15                                                  */
    double damp_strength;         /* DD damping, default 0.75                                    */
    double schwarz;               /* J/K screening threshold (default 1e-14)                     */
    int solver[8];                /* per method: QB_DIIS_* coefficient solver (default LBFGS)    */
} qb_scf_config;

typedef struct {
    double E_elec;                /* electronic energy (Ha)                                      */
    double E_nuc;                 /* nuclear repulsion (Ha)                                      */
    int converged;                /* 0 no, 1 yes, 2 converged to an oscillation                  */
    int steps;
    double dE, rms_dD, rms_FDS;   /* last-step convergence indicators                            */
    double* C;                    /* optional outputs (caller-allocated, nspin * nfun^2 / nfun)  */
    double* D;
    double* F;
    double* eps;
} qb_scf_result;

void qb_scf_config_default(qb_scf_config* cfg);
int qb_run_hartree_fock(qb_ctx* ctx, const qb_basis* basis, int nnuc, const double* Z, const double* R,
                        int n_alpha, int n_beta, const qb_scf_config* cfg, qb_scf_result* res);

/* Batched closed-shell Hartree–Fock over many independent molecules in one call.
 * The reference solves one molecule per runHartreeFock (src/HartreeFock.jl:953-1046);
 * this runs hundreds of them together: integrals of all molecules once (screened ERI
 * blocks stored on the device), then every SCF iteration of every molecule in one launch
 * of a CUDA graph whose conditional while-node repeats (digest, step) passes until no
 * molecule iterates.  Per molecule: a flattened basis of s and p Cartesian shells
 * (1 <= nfun <= 256), nnuc[m] nuclei (charges and positions concatenated over molecules in
 * Z and R), nocc[m] doubly occupied orbitals.  Core-Hamiltonian guess (or initial_density),
 * symmetric orthogonalisation, then runHartreeFockCore's method sequence
 * (src/HartreeFock.jl:1049-1228) per molecule: nmethod = 0 runs one DIIS method with exact
 * (Lagrange-multiplier) coefficients, converged when |dE| <= conv_energy and
 * RMS(dD_total) <= conv_density; nmethod >= 1 runs the given methods, thresholds and
 * coefficient solvers with the reference's convergence, oscillation and early-stop rules,
 * e.g. its default SCFconfig (DD, ADIIS, DIIS) with L-BFGS-B.  energy[m] receives the
 * electronic energy (add the nuclear repulsion for the total). */
typedef struct {
    double conv_energy;     /* default 1e-10 Ha */
    double conv_density;    /* default 1e-8 */
    int max_iter;           /* default 200 */
    int diis_size;          /* 1..15, default 15 (1 = no extrapolation) */
    double schwarz;         /* stored-integral screening Q_ab Q_cd >= schwarz, default 1e-14 */
    int iters_per_graph;    /* SCF iterations per CUDA-graph launch, default 4 */
    const double* initial_density;  /* NULL: core-Hamiltonian guess; else per-spin densities
                                       of all molecules, nfun x nfun each (column-major),
                                       concatenated; host or device memory */
    int eigensolver;        /* 0 (default): occupied eigenvectors by Householder tridiagonalisation,
                               bisection and inverse iteration; 1: Jacobi over all eigenvectors */
    int jacobi_sweeps;      /* eigensolver 1: sweeps per SCF iteration (eigenvectors carry over from
                               the previous iteration); 0: until converged (default) */
    int fallback_iter;      /* with initial_density: a molecule not converged after this many
                               iterations restarts from the core-Hamiltonian guess in the same call
                               (the iterations of both attempts count against max_iter); 0: never
                               (default) */
    int nmethod;            /* 0 (default): the single DIIS method above; 1..8: the strategy below */
    int method[8];          /* QB_SCF_* per method (as qb_scf_config)                            */
    double interval[8];     /* per-method thresholds; the last converges                         */
    int solver[8];          /* QB_DIIS_* per method (default LBFGS)                               */
    double secondary_ratio[2];   /* RMS(FDS-SDF) and RMS(dD) ratios (default 1000, 1000)         */
    double oscillate_threshold;  /* default 5e-6                                                 */
    int early_stop;         /* default 1                                                          */
    double damp_strength;   /* DD damping, default 0.75                                           */
    int digest_chunk;       /* stored quartets per digest block of a molecule with much work in a
                               class (a quarter of it for the others); 0 (default): chosen by timing
                               on the batch                                                          */
} qb_batch_config;

typedef struct {
    double* energy;         /* nmol electronic energies (caller-allocated, may be NULL) */
    int* iterations;        /* nmol */
    int* converged;         /* nmol: 1 if converged */
    int* jacobi_sweeps;     /* nmol: Jacobi sweeps summed over the iterations */
    double ms_integrals;    /* device time: one-body, pairs, Schwarz, stored ERIs, orthogonalisation */
    double ms_scf;          /* device time of the SCF iterations */
    int64_t quartets;       /* stored shell quartets */
    int64_t prim_quartets;  /* primitive quartets evaluated for them */
    int64_t eri_doubles;    /* stored integrals */
    int graph_launches;     /* 1: the whole iteration ran as one graph launch */
    double* density;        /* NULL or room for the final per-spin densities, concatenated */
    int* restarted;         /* NULL or nmol: 1 if the molecule restarted from the core-Hamiltonian guess */
    int digest_chunk;       /* quartets per digest block chosen by timing on this batch (molecules with
                               little work in a class use a quarter of it) */
} qb_batch_result;

void qb_batch_config_default(qb_batch_config* cfg);
int qb_run_rhf_batched(qb_ctx* ctx, int nmol, const qb_basis* bases, const int* nnuc, const double* Z,
                       const double* R, const int* nocc, const qb_batch_config* cfg, qb_batch_result* res);

/* One DIIS coefficient solve on the device, the step of xDIIScore! (src/HartreeFock.jl:1322-1331)
 * that constraintSolver! (:1479-1487) performs: minimise v.c/s + c^T B c/(2 s^2), s = sum c
 * (genxDIISf, :1398-1404), with c >= 0 when convex != 0 (EDIIS / ADIIS).  B is m x m
 * column-major, v has m entries (NULL = zeros, as DIIS), 1 <= m <= 15; c (m) is the starting
 * point on entry (the reference carries the previous solution over) and the normalised
 * coefficients on return.  solver: QB_DIIS_LBFGS, QB_DIIS_SPGB or QB_DIIS_LCM.  iterations
 * (may be NULL) receives the L-BFGS-B iteration count. */
int qb_diis_coefficients(qb_ctx* ctx, int solver, int convex, int m, const double* B, const double* v, double* c,
                         int* iterations);

/* Measured FP64 FMA throughput of this device (TFLOP/s), the FP64 roofline denominator. */
int qb_fp64_peak(qb_ctx* ctx, double* tflops);
/* Measured FP64 tensor-core throughput of this device (mma.sync m8n8k4 f64, TFLOP/s), for
 * comparison with qb_fp64_peak (no counterpart in the reference). */
int qb_fp64_dmma_peak(qb_ctx* ctx, double* tflops);

/* Allocation-free direct J/K (no counterpart in the reference).
 * For callers that cannot allocate device memory themselves (code inside a host
 * framework that owns every device allocation, or code that must not allocate
 * between graph captures): computes the same J and K as qb_jk with the generic
 * per-function kernels and calls no cudaMalloc / cudaFree.  Everything is device
 * memory owned by the caller: `dbasis` holds DEVICE pointers (fun_ptr, center, ijk,
 * alpha, weight), dD is the nfun x nfun density, dJ / dK receive the results;
 * `stream` is a cudaStream_t (NULL = legacy default stream).  No Schwarz screening.
 *  - Limit: nfun <= 512; larger bases return QB_ERR_DIM before touching any pointer.
 *  - Scratch: a file-scope device array of 4 MiB (+ a 2.1 MiB Boys table) held by
 *    every GPU that loads the library until exit.  The first call on a device does
 *    the set-up (resolves the arrays' device addresses, uploads the Boys table) and
 *    must come before any stream capture on that device.
 *  - Every call shares the array: calls that overlap on the GPU (other streams,
 *    other host threads) race and corrupt each other's results.
 *  - Bad basis data returns QB_ERR_ARG (pointer layout), QB_ERR_UNSUPPORTED
 *    (angular momentum > 12) or QB_ERR_DOMAIN (exponent <= 0).  No context, so no
 *    qb_last_error() message.
 *  - The call waits on `stream` three times (after each of the two input checks and for
 *    the final status), so it returns with its work finished.
 *  - Cost: it evaluates every canonical function quartet (about nfun^4/8) without
 *    screening, far more work than qb_jk's shell-quartet kernels: measured on a GB300 with
 *    s/p/d bases, 1.8 s per call at nfun = 100 and 26 s at nfun = 200 (qb_jk, unscreened:
 *    0.05 s and 0.16 s).  It suits small bases. */
int qb_jk_noalloc(const qb_basis* dbasis, const double* dD, double* dJ, double* dK, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* QUIQBOX_GB300_H */

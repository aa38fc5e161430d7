/*
 * ls_dafmm.h - C ABI of the GB300 DAFMM matvec + GMRES library
 * (liblsdafmm.so, package lippmann_schwinger_solver_gb300).
 *
 * Drop-in boundary for the hot path of vaishna77/Lippmann_Schwinger_Solver:
 * the operator that the reference's GMRES drives through the duck-typed
 * `MatVecProduct(Vec&, Vec&)` member. Every entry point below names the
 * reference interface it replaces. Plain pointers and sizes only; complex
 * vectors are interleaved (re, im) doubles in the reference's leaf order
 * (depth-first leaves, 36 Chebyshev nodes per leaf, node = row * n + col).
 * All functions return LS_OK (0) or a negative LS_E_* code and never exit
 * the process; ls_last_error() describes the last failure on this thread.
 * Threading: an operator serves one call at a time (its device buffers and
 * stream are its own); distinct operators may be created, solved and
 * destroyed from different threads at the same time.
 */
#ifndef LS_DAFMM_H
#define LS_DAFMM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int ls_status;
#define LS_OK 0
#define LS_E_INVALID (-1)     /* bad argument or configuration */
#define LS_E_CUDA (-2)        /* a CUDA call failed */
#define LS_E_NOMEM (-3)       /* host or device allocation failed */
#define LS_E_NOT_CONVERGED (-4)
#define LS_E_STATE (-5)       /* handle used in the wrong state */
#define LS_E_TIMEOUT (-6)     /* a bounded device wait gave up */

#define LS_MAX_BUMPS 8
#define LS_ASSEMBLE_STAGES 6

/* Precision of the operator blocks and their accumulation. */
#define LS_PREC_F64 0
#define LS_PREC_F32 1

/* Kernels behind the FP64 entry points (ls_matvec, ls_matvec_host, ls_gmres,
 * ls_gmres_restarted, the FP64 residual of ls_gmres_mixed, ls_time_matvec
 * with LS_PREC_F64). NATIVE: FP64 arithmetic. DOUBLE_FLOAT: every complex
 * double held as an FP32 hi/lo pair (48-bit significand) and multiplied and
 * summed with error-free FP32 transformations; same operator, same inputs
 * and outputs; measured relative L2 distance from the native kernels 1e-14
 * (Lippmann-Schwinger operator) to 4e-12 (bare Helmholtz operator). */
#define LS_F64_NATIVE 0
#define LS_F64_DOUBLE_FLOAT 1

/*
 * Problem description. Replaces the positional argv of GMRES/GMRES.cpp:321-333
 * (main), the inputsToDFMM struct (GMRES/GMRES.cpp:129-138), the global
 * `kappa` (GMRES/G_FMM2DTree.hpp:3) and the contrast plugin selected by the
 * global `Qchoice` (GMRES/GMRES.cpp:4, 100-117).
 */
typedef struct {
  int nCones_LFR;          /* cones of a box at the finest HFR level (16) */
  int nChebNodes;          /* Chebyshev nodes per leaf per direction (6) */
  int yes2DFMM;            /* 1: directional DAFMM, 0: AFMM (level_LFR = 2) */
  int TOL_POW;             /* NCA tolerance 10^-TOL_POW */
  int degreeOfBases;       /* 6 -> 21 Chebyshev basis polynomials */
  int nLevelsUniform;      /* depth of the uniform quadtree (3..10) */
  int Qchoice;             /* 0..5 reference contrasts, 6 = Gaussian bumps */
  int findPhi;             /* 1: I + k^2 q G (LS operator); 0: bare G */
  int reference_rounding;  /* 1: M and near blocks rounded to 6 significant
                              digits, as the reference's text cache does */
  int n_bumps;             /* Qchoice 6: q(x) = sum_k a_k exp(-|x-c_k|^2/w_k^2) */
  double L;                /* half side of the square domain */
  double kappa;            /* wavenumber */
  double bump_cx[LS_MAX_BUMPS];
  double bump_cy[LS_MAX_BUMPS];
  double bump_a[LS_MAX_BUMPS];
  double bump_w[LS_MAX_BUMPS];
  /* Tree: 0 (zero-initialised) = the uniform quadtree of nLevelsUniform
   * levels (createUniformTree, G_FMM2DTree.hpp:917); 1 = the adaptive
   * quadtree of the reference's default path (createAdaptiveTree +
   * makeLevelRestriction_Tree, GMRES/GMRES.cpp:165-166): boxes split until
   * q is resolved to 10^-treeAdaptivity and no box spans more than one
   * wavelength, then 2:1 balanced. Adaptive operators support the FP64 and
   * FP32 matvecs, the GMRES solvers and the batched ones; the
   * allocation-free, interpolation and network entry points return
   * LS_E_STATE for them. */
  int tree_adaptive;
  int treeAdaptivity;
  /* 1: the precomputation quadratures (far moments M and near blocks) run on
   * the operator's GPU; 0 (zero-initialised, the default): on the host
   * cores, as the reference does. The GPU's values differ from the host's in
   * the last bits; M entries that are zero by symmetry then carry other
   * round-off, and NCA pivots among entries at that noise level change, so
   * the operator is no longer the oracle's bit for bit (its matvec stays
   * within about 1e-7 of it on the tested trees). Operators assembled
   * without a device always integrate on the host. */
  int precompute_on_gpu;
  /* Far-field assembly of a uniform tree (getMatrixEntry,
   * G_FMM2DTree.hpp:603-658; ACA_only_nodes, GMRES/ACA.hpp:253-481):
   * 0 (the default): on the host cores, entries from a cache of Hankel sums
   * filled on demand, bit-exact with the reference's algorithm;
   * 1: the far-field sums of every distinct relative position are tabulated
   * on the operator's GPU (on the host cores when it has no device) and the
   * host's NCA and block fills read them from that table;
   * 2: as 1, and the NCA skeleton search of every box runs on the GPU as
   * well (one thread block per box and direction; the host redoes any box
   * whose rank passes the GPU's capacity);
   * 3: as 2, and the M2L blocks (Assemble_LFR_M2L / Assemble_HFR_M2L,
   * G_FMM2DTree.hpp:2502, 3829) are filled from the table straight into the
   * device operator's tiles, never formed on the host (without a device, on
   * the host from the same table).
   * GPU values differ from the host's in the last bits, which moves NCA
   * pivots among candidates equal in magnitude up to such bits (mirror-image
   * positions of a uniform tree): the skeletons are other valid choices, and
   * the matvec moves by less than the host-assembled operator itself moves
   * when the NCA tolerance is tightened tenfold. Adaptive trees ignore it,
   * and so do trees whose table would pass 4 GB (the x and y offsets of a
   * level-8 tree give about 14 GB; level 7: 2.9 GB): those assemble on the
   * default path. */
  int far_on_gpu;
} ls_config;

typedef struct {
  int N;                   /* unknowns = leaves * nChebNodes^2 */
  int n_leaves;
  int n_levels;
  int level_LFR;
  int rank;                /* nChebNodes^2 */
  long long far_entries;   /* complex entries of all M2M/M2L/L2L blocks */
  long long near_entries;  /* complex entries of the near blocks (shared) */
  long long matvec_bytes;  /* algorithmic HBM bytes of one FP64 matvec */
  long long matvec_flops;  /* real flops of one matvec */
  long long device_bytes;  /* device memory held by the operator */
  double assemble_seconds; /* host assembly wall time */
  int max_rank;            /* largest NCA skeleton */
  int n_kernels_per_matvec;/* CUDA kernel launches in one matvec */
  long long m2l_entries;   /* complex entries of the M2L blocks */
  long long m2l_bytes;     /* algorithmic bytes of the M2L kernel (FP64) */
  long long m2l_flops;     /* real flops of the M2L kernel */
  /* Host assembly wall time by stage, seconds: [0] tree geometry and leaf
     quadrature, [1] precomputations (Chebyshev fits, near blocks, leaf
     multipoles), [2] interaction lists, [3] NCA skeletons of every level,
     [4] user checks, [5] block fill, folding and tile packing. */
  double assemble_stage_seconds[LS_ASSEMBLE_STAGES];
} ls_op_info_t;

typedef struct ls_op ls_op;

/*
 * Builds the tree, interaction lists, cones, precomputations and NCA
 * skeletons, assembles every block and uploads the operator to `device`.
 * Replaces DFMM::DFMM + DFMM::FMMTreeInitialisation (GMRES/GMRES.cpp:152-199)
 * for uniform trees (createUniformTree, GMRES/G_FMM2DTree.hpp:917).
 * device < 0 assembles on the host only: geometry, precomputations and
 * skeletons can be inspected, every device call returns LS_E_STATE.
 */
ls_status ls_op_create(const ls_config* cfg, int device, ls_op** out);
ls_status ls_op_destroy(ls_op* op);
ls_status ls_op_info(const ls_op* op, ls_op_info_t* out);

/* Chebyshev grid points (N x 2) in the operator's order; replaces
 * DFMM::gridPoints (GMRES/GMRES.cpp:145, G_FMM2DTree.hpp:1150-1163). */
ls_status ls_op_points(const ls_op* op, double* xy);
/* q(x_i) at the grid points; userkernel::ContrastFunction (GMRES/GMRES.cpp:104). */
ls_status ls_op_contrast(const ls_op* op, double* q);
/* b_i = -kappa^2 q(x_i) exp(i kappa x_i1); userkernel::RHSFunction (GMRES/GMRES.cpp:122-125). */
ls_status ls_op_rhs(const ls_op* op, double* b);
/* Right-hand sides of n incidence directions: column t of b (N x n complex,
 * column major) is -kappa^2 q(x_i) exp(i kappa (x_i1 cos th_t + x_i2 sin th_t)),
 * the reference's RHSFunction (GMRES/GMRES.cpp:122-125) turned by th_t
 * (th_t = 0 gives ls_op_rhs bit for bit). Host threads; the many-direction
 * workload forms its right-hand sides with it. */
ls_status ls_op_rhs_angles(const ls_op* op, const double* thetas, int n, double* b);

/*
 * y = A x on the device. x and y are device pointers to N complex values
 * (2N doubles). Replaces DFMM::MatVecProduct (GMRES/GMRES.cpp:201-254).
 * `stream` is a cudaStream_t (NULL = the operator's own stream). The call
 * is asynchronous with respect to the host.
 */
ls_status ls_matvec(ls_op* op, const double* x, double* y, void* stream);
/* Same product with FP32 blocks and FP32 accumulation (x, y stay FP64 on
 * the boundary). Requires ls_op_enable_f32(). */
ls_status ls_matvec_f32(ls_op* op, const double* x, double* y, void* stream);
ls_status ls_op_enable_f32(ls_op* op);
/* Selects the kernels of the FP64 entry points (LS_F64_*). The first switch
 * to LS_F64_DOUBLE_FLOAT builds the hi/lo copies of the operator on the
 * device (as much memory again as the FP64 blocks). No counterpart in the
 * reference, whose arithmetic is FP64 throughout. */
ls_status ls_op_set_f64_kernels(ls_op* op, int kernels);
/*
 * Allocation-free variant of ls_matvec. No counterpart in the reference.
 * For callers that may not allocate device memory while they run (for
 * example a solver inside a framework whose caching allocator owns the
 * device heap): the matvec's scratch (skeleton charges and potentials) is
 * taken from a fixed device array of LS_STATIC_SCRATCH_ELEMS complex
 * doubles (16 MiB) that every GPU loading the library reserves until exit;
 * nothing is allocated or freed per call. x, y and the operator stay
 * caller-provided as in ls_matvec. Operators that need more scratch are
 * rejected with LS_E_INVALID (checked before anything else, so a host-only
 * operator gets the same answer). It always runs the native FP64 kernels,
 * with the unfactored near-field blocks, whatever ls_op_set_f64_kernels
 * selected. The first call on a device looks up the array's device address
 * in the current CUDA context (make it before any stream capture); a call
 * after cudaDeviceReset looks it up again. All calls share the array:
 * calls that overlap on the GPU race and must be serialised by the caller.
 */
#define LS_STATIC_SCRATCH_ELEMS (1LL << 20)
ls_status ls_matvec_noalloc(ls_op* op, const double* x, double* y, void* stream);
/* Host-buffer convenience: copies x in, runs ls_matvec, copies y out, syncs.
 * This is the call a reference-style driver makes (Vec in, Vec out). When x
 * and y are distinct page-locked buffers (cudaMallocHost, cudaHostRegister)
 * the matvec reads x from and writes y to host memory directly, without
 * separate copies; the result is the same. */
ls_status ls_matvec_host(ls_op* op, const double* x, double* y);

/*
 * Tolerance-stopped GMRES with Givens rotations, x0 = 0; replaces
 * classGMRES::gmres (GMRES_Hybrid/include/gmres.hpp:54-119), with the
 * conjugate-linear inner product and unitary complex rotations. b and x are
 * HOST buffers of N complex values; history receives |r_k|/|b| estimates
 * (max_iter + 1 entries, may be NULL). Returns LS_E_NOT_CONVERGED (with x
 * filled) when max_iter is reached first.
 */
ls_status ls_gmres(ls_op* op, const double* b, int max_iter, double tol, double* x,
                   double* history, int* n_iter, double* rel_residual);
/* Fixed-m restarted GMRES (GMRES/GMRES.cpp:257-319, RestartedGMRES). */
ls_status ls_gmres_restarted(ls_op* op, const double* b, int m, int restarts, double* x);

/* Mixed precision: FP64 iterative refinement whose inner GMRES solves use
 * the FP32 operator (needs ls_op_enable_f32). Stops on the FP64 true
 * residual. The inner Krylov basis, its Gram-Schmidt and the Givens
 * rotations are FP64 unless ls_op_set_inner_basis selected FP32. */
ls_status ls_gmres_mixed(ls_op* op, const double* b, int max_outer, int inner_iter,
                         double tol, double* x, double* history, int* n_matvec,
                         double* rel_residual);
/* Element type of the inner Krylov basis of ls_gmres_mixed and
 * ls_fgmres_nn. LS_INNER_BASIS_F64 (default): Arnoldi vectors, classical
 * Gram-Schmidt and Givens in FP64 around the FP32 operator apply;
 * LS_INNER_BASIS_F32: the basis and its orthogonalisation in FP32 as well
 * (half the basis memory and traffic). No counterpart in the reference. */
#define LS_INNER_BASIS_F64 0
#define LS_INNER_BASIS_F32 1
ls_status ls_op_set_inner_basis(ls_op* op, int basis);

/*
 * Many right-hand sides on one operator (e.g. the incident fields of many
 * directions on one scatterer). No single counterpart in the reference,
 * which runs one GMRES per right-hand side (GMRES/GMRES.cpp:336-470).
 * Solves A x_j = b_j for j < nrhs with the mixed-precision refinement of
 * ls_gmres_mixed, kBatchRhs (8) columns at a time: the inner FP32 GMRES of
 * the columns share every operator apply, and each column stops on its own
 * FP64 true residual. B and X are host arrays of nrhs columns of N complex
 * values (column j at 2 * N * j doubles). n_matvec counts FP32 block
 * applies plus FP64 residual products; rel_residuals (nrhs, may be NULL)
 * gets each column's final FP64 relative residual. Needs
 * ls_op_enable_f32(); LS_E_NOT_CONVERGED when a column misses tol.
 */
ls_status ls_gmres_mixed_batched(ls_op* op, int nrhs, const double* B, int max_outer, int inner_iter, double tol,
                                 double* X, int* n_matvec, double* rel_residuals);
/* Right-hand sides per block of ls_gmres_mixed_batched: 64 (the default)
 * carries each block through the FP32 operator on the tensor cores
 * (tcgen05, TF32 inputs split into three products for FP32 accuracy, FP32
 * accumulation), whose tensor-core form is built on the device on first
 * use (about twice the FP32 blocks' memory); 8 uses the CUDA-core block
 * kernels. A tensor-core pipeline wait that gives up returns LS_E_TIMEOUT.
 * No counterpart in the reference. */
ls_status ls_op_set_batch_width(ls_op* op, int width);
/* Y = A32 X for nrhs columns of N complex values (host arrays, column j at
 * 2 * N * j doubles), 64 columns per pass on the tensor cores: the block
 * apply of ls_gmres_mixed_batched with width 64. Needs ls_op_enable_f32.
 * No counterpart in the reference. */
ls_status ls_matvec_f32_many(ls_op* op, int nrhs, const double* X, double* Y);
/* Mean ms of one FP32 block apply of `width` resident right-hand sides (8:
 * CUDA-core block kernels, 64: tensor cores), CUDA events on the
 * operator's stream after `warmup` untimed applies. No counterpart in the
 * reference. */
ls_status ls_time_block_apply(ls_op* op, int width, int warmup, int iters, float* ms);
/* Stages (16 complex columns of one block) of one 64-wide tensor-core block
 * apply, all phases; 0 before the tensor-core form is built (by the first
 * 64-wide apply). Each stage is 12 MMAs. No counterpart in the reference. */
ls_status ls_op_tc_stages(const ls_op* op, long long* stages);
/* The bounded-wait path of the tensor-core kernels, on its own: one CTA
 * allocates tensor memory, waits `polls` polls (1 .. 1e8) on an mbarrier
 * that nothing arrives on, records that the wait gave up as the kernels do
 * (the flag behind LS_E_TIMEOUT), frees the tensor memory and exits; writes
 * *gave_up = 1. The context stays usable. For tests of failure detection
 * without a GPU fault. No counterpart in the reference. */
ls_status ls_tc_wait_probe(int device, long long polls, int* gave_up);
/* Times `iters` device matvecs (inputs resident) with CUDA events on the
 * operator's stream after `warmup` untimed ones; writes the mean ms per
 * matvec and the mean ms of the dominant kernel (M2L). precision: LS_PREC_*. */
ls_status ls_time_matvec(ls_op* op, int precision, int warmup, int iters, float* ms_matvec,
                         float* ms_m2l);

/* Same timing split by phase, each the mean over `iters` matvecs, in ms:
 * ms[0] whole matvec, ms[1] load of x and the upward (M2M) phases, ms[2] M2L,
 * ms[3] downward (L2L) phases, ms[4] near field and output. The events
 * between the phases stop consecutive kernels from overlapping, so ms[1..4]
 * add up to slightly more than an unmarked matvec. No counterpart in the
 * reference. */
ls_status ls_time_matvec_phases(ls_op* op, int precision, int warmup, int iters, float* ms);

/*
 * Measured arithmetic peak of `device`: a kernel of independent fused
 * multiply-add chains (2 flops each) over every SM, best of a few timed
 * launches with CUDA events. kind 0: FP64 (DFMA), 1: FP32 (FFMA). Writes
 * TFLOP/s. The denominator of the FP64-pipe roofline of the native kernels.
 * No counterpart in the reference.
 */
ls_status ls_measure_fma_peak(int device, int kind, double* tflops);
/*
 * Issue cost of one TF32 tensor-core MMA (M = 128, N = n, K = 8) on `device`:
 * one CTA per SM issues 512 back-to-back MMAs into one accumulator; writes
 * the mean SM cycles per MMA over the SMs (second of two launches). n is a
 * multiple of 16 in [16, 256]. Below n = 128 the cost does not depend on n:
 * the floor of the tensor-core block apply (12 MMAs per stage). No
 * counterpart in the reference.
 */
ls_status ls_measure_mma_issue(int device, int n, double* clocks_per_mma);

/*
 * Density at arbitrary points by the reference's Chebyshev-Q+ interpolation
 * (GMRES_Hybrid/LippmannSchwinger/main/hybridTrueValidation_gmres.cpp:
 * 187-219, the "Psi_non_grid" loop): in the leaf that contains (x, y),
 * c = Q^+ phi_leaf and psi = sum_l c_l T_a(l)(x') T_b(l)(y') with
 * x' = (x - centre) / radius. Host buffers: xy (npts x 2), phi (N complex),
 * psi (npts complex). Points outside [-L, L]^2 give LS_E_INVALID (the
 * reference runs off the end of its leaf list there); points on the upper
 * edges belong to the last leaf. Works for host-only operators.
 */
ls_status ls_op_interpolate(const ls_op* op, int npts, const double* xy, const double* phi, double* psi);

/* Writes n complex values to `path`, one per line as "(re,im)" with six
 * significant digits: the text of the reference's result files
 * (GMRES/GMRES.cpp:391-397, `myfile0 << Phi(l) << endl`). */
ls_status ls_write_result(const char* path, int n, const double* v);

/* Flattened NCA skeletons (one record per tree node: level, box, cone,
 * out_active, in_active, then counted lists out-charge, out-check,
 * in-charge, in-check, user-check). Returns the length; buf may be NULL. */
long ls_op_skeleton_dump(const ls_op* op, int* buf, long cap);
/* Leaf-level far-field moments M (rank x 31, complex) and colleague near
 * blocks (9 x rank x rank, complex, row major) as used by the matvec. */
ls_status ls_op_precomputations(const ls_op* op, double* M, double* near);

/*
 * Launch mode of the matvec and Krylov kernel chains. No counterpart in the
 * reference (a CPU code). 1 (the default): programmatic dependent launch,
 * each kernel scheduled while its predecessor runs and waiting in hardware
 * for its results; 0: plain stream-ordered launches. Results are bitwise
 * identical in both modes. LS_PDL=0 in the environment selects 0 at load.
 * Process-wide; applies to launches queued after the call.
 */
ls_status ls_set_pdl(int on);
int ls_get_pdl(void);
/*
 * Near-field schedule of the native FP64 matvec on uniform trees. No
 * counterpart in the reference. 1 (the default): the near field (Q+ x per
 * leaf and the factored colleague blocks) runs on a second stream of the
 * same priority beside the upward, M2L and downward phases, whose latency-bound
 * launches leave FP64 issue slots free, and one kernel adds it to the
 * potentials at the end; 0: after them, in one stream. Results are bitwise
 * identical in both modes. LS_NEAR_OVERLAP=0 in the environment selects 0 at
 * load. Process-wide; applies to matvecs queued after the call. Phase timing
 * (ls_time_matvec_phases) always runs the near field after the far field.
 */
ls_status ls_set_near_overlap(int on);
int ls_get_near_overlap(void);

/*
 * Cache of the assembly's precomputations (the far moments M of a leaf size
 * and the near-field blocks), replacing the reference's text files
 * (writeMToFile / writeNeighborInteractionsForLevel and their readers,
 * G_FMM2DTree.hpp:1264-1270, 1868-1950), which hold the values at 6
 * significant digits and are recomputed on every run. A record holds the
 * exact values an assembly computed and is keyed on every input they depend
 * on (kappa, the leaf radii and neighbour offsets, nChebNodes,
 * degreeOfBases, reference_rounding, host or GPU integration), so an
 * assembly that reads it is the same bit for bit. dir NULL: off (the
 * default); "": records kept in memory for the process; a directory: also
 * stored there as binary files (one per record, shared between processes;
 * a file that does not match its key is ignored; a directory that cannot
 * be written costs only the files). Records held in memory are capped at
 * 2 GB, past which they are dropped (the files still serve). Process-wide;
 * setting it drops the records held in memory. ls_precompute_cache_stats: records
 * found and not found since the process started.
 */
ls_status ls_set_precompute_cache(const char* dir);
ls_status ls_precompute_cache_stats(long long* hits, long long* misses);

const char* ls_last_error(void);
const char* ls_version(void);

#ifdef __cplusplus
}
#endif
#endif

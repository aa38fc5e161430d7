/*
 * ls_fno.h - C ABI of the learned preconditioner (liblsdafmm.so).
 *
 * A spectral neural operator (Fourier neural operator) on a G x G grid over
 * the scatterer's square [-L, L]^2 maps the contrast and a right-hand side f
 * (the incident field weighted by the contrast, -kappa^2 q u_inc, or any
 * residual) to the multiple-scattering part of the scattered density,
 * A^-1 f - f, so that M(f) = f + net(f) approximates A^-1 f. M is the
 * initial guess and the nonlinear right preconditioner of the flexible
 * mixed-precision GMRES (ls_fgmres_nn); the net is trained only on
 * solutions that the plain solver produces. No counterpart in the reference, whose
 * solver is unpreconditioned GMRES (GMRES/GMRES.cpp:257-319); the grid
 * resampling follows the reference's Chebyshev-Q+ interpolation
 * (GMRES_Hybrid/LippmannSchwinger/main/hybridTrueValidation_gmres.cpp:187-219).
 *
 * Layouts. Grid point g = ix * G + iy sits at
 * (x, y) = L (-1 + (2 ix + 1) / G, -1 + (2 iy + 1) / G). Network inputs are
 * [batch][G*G][6] floats: q, Re f, Im f, kappa / 40, x / L, y / L; outputs
 * [batch][G*G][2] (Re, Im). The flat FP32 parameter vector holds, in order:
 * lift weight [32][6] and bias [32]; per Fourier layer the spectral weights
 * [2M][M][32 in][32 out] complex (kx = 0..M-1 then G-M..G-1; ky = 0..M-1),
 * the pointwise weight [32 out][32 in] and bias [32]; projection
 * [proj][32], [proj], [2][proj], [2].
 * All device pointers are on the net's (operator's) device. `stream` is the
 * cudaStream_t the work is queued on, NULL being CUDA's default stream, so
 * that buffers written on the caller's stream are read in order. A net keeps
 * its activations in its own buffers: use one net from one stream at a time.
 */
#ifndef LS_FNO_H
#define LS_FNO_H

#include "ls_dafmm.h"

#ifdef __cplusplus
extern "C" {
#endif

#define LS_FNO_IN_CHANNELS 6
#define LS_FNO_OUT_CHANNELS 2
#define LS_FNO_WIDTH 32
#define LS_FNO_MAX_BATCH 64

typedef struct {
  int grid;        /* G: power of two in [8, 256] (128) */
  int modes;       /* M: kept Fourier modes per axis, 2 M <= G, M <= 32 (24) */
  int layers;      /* Fourier layers, 1..8 (4) */
  int proj_width;  /* hidden width of the output projection: 32, 64, 96 or 128 (128) */
} ls_fno_config;

typedef struct ls_fno ls_fno;

ls_status ls_fno_create(const ls_fno_config* cfg, int device, unsigned long long seed, ls_fno** out);
ls_status ls_fno_destroy(ls_fno* net);
ls_status ls_fno_num_params(const ls_fno* net, long long* n);
ls_status ls_fno_get_params(const ls_fno* net, float* host);
ls_status ls_fno_set_params(ls_fno* net, const float* host);
/* Gradients of the last ls_fno_loss_grad (same layout as the parameters). */
ls_status ls_fno_get_grads(const ls_fno* net, float* host);

/* out = net(in) for `batch` samples (device buffers). */
ls_status ls_fno_forward(ls_fno* net, int batch, const float* in, float* out, void* stream);
/* Forward, loss = mean_b |out_b - target_b|^2 / |target_b|^2, and backward:
 * the gradients overwrite the net's gradient buffer. loss (host) may be
 * NULL; when given, the call waits for the stream and stores the loss. */
ls_status ls_fno_loss_grad(ls_fno* net, int batch, const float* in, const float* target, float* loss, void* stream);
/* One Adam step on the stored gradients (bias-corrected). */
ls_status ls_fno_adam_step(ls_fno* net, float lr, float beta1, float beta2, float eps, void* stream);

/*
 * Training batch from solved fields (device buffers). For sample b, with
 * s = scatterer[b] and complex coefficients c = coef[b][0:n_basis]:
 *   f = sum_m c_m F[s][m],  t = sum_m c_m PHI[s][m]
 * (F, PHI: [n_scatterers][n_basis][G*G] complex), both divided by the RMS
 * of f; in[b] = (Q[s], Re f, Im f, kappa[s], x / L, y / L), target[b] = t.
 * kappa[s] is the kappa channel value (kappa / 40). By linearity of the
 * solution in the right-hand side, t solves the problem with data f. A
 * scatterer index outside [0, n_scatterers) yields an all-zero sample.
 */
ls_status ls_fno_make_batch(ls_fno* net, int batch, int n_basis, int n_scatterers, const float* F, const float* PHI,
                            const float* Q, const float* kappa, const int* scatterer, const float* coef, float* in,
                            float* target, void* stream);

/* Nodes -> grid: out[v][G*G] (complex FP32) from nvec FP64 vectors x[v][N]
 * (device buffers; queued on `stream`, NULL = CUDA's default stream). */
ls_status ls_op_grid_sample(ls_op* op, int grid, int nvec, const double* x, float* out, void* stream);
/* Host: weight rows [G*G][rank] and leaf [G*G] of the nodes -> grid map
 * (works for host-only operators). */
ls_status ls_op_grid_weights(const ls_op* op, int grid, float* w, int* leaf);
/* Host: q at the G x G grid points. */
ls_status ls_op_grid_contrast(const ls_op* op, int grid, float* q);

#define LS_NN_GUESS 1    /* start from x0 = net(b) */
#define LS_NN_PRECOND 2  /* right-precondition the inner FP32 GMRES with the net */

typedef struct {
  int n_matvec;          /* FP32 operator applies + FP64 residual products */
  int n_precond;         /* network applications */
  int outer;             /* FP64 refinement steps */
  int fell_back;         /* 1: the net was dropped after a step that did not halve the residual */
  double guess_residual; /* |b - A x0| / |b| of the initial guess (1 without one) */
  double rel_residual;   /* final FP64 |b - A x| / |b| */
} ls_nn_report;

/*
 * Mixed-precision flexible GMRES with the network: FP64 refinement around
 * inner FP32 flexible GMRES on the FP32 operator, right-preconditioned by
 * the net (flags & LS_NN_PRECOND), starting from net(b) (flags &
 * LS_NN_GUESS). The stopping test is always the FP64 true residual. The net
 * preconditions only outer steps that must reduce the residual by more than
 * 1e3 (looser targets take a few plain steps, cheaper than network
 * applications); it is dropped, returning the solve to plain GMRES, when
 * an outer step (at most 24 preconditioned inner steps) does not halve the
 * residual; a guess worse than x0 = 0 is discarded.
 * With flags = 0 this is ls_gmres_mixed. b, x: host, N complex. history
 * (max_outer + 2 entries, may be NULL) gets the FP64 residual after the
 * guess and after each outer step. Needs ls_op_enable_f32(); net and
 * operator on the same device. LS_E_NOT_CONVERGED when tol is missed.
 */
ls_status ls_fgmres_nn(ls_op* op, ls_fno* net, const double* b, int flags, int max_outer, int inner_iter, double tol,
                       double* x, double* history, ls_nn_report* report);

#ifdef __cplusplus
}
#endif
#endif

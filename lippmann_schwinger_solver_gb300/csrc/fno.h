// Spectral neural operator (Fourier neural operator, FNO) on a square grid,
// with hand-written forward, backward and Adam kernels (fno.cu).
//
// Network: 6 input channels per grid point (contrast q, Re f, Im f, kappa/40,
// x/L, y/L) -> lift to 32 channels -> n_layers Fourier layers
//   z = irfft2(W_spec . rfft2(h)[kept modes]) + W h + b,  h' = GELU(z)
//   (no activation after the last layer)
// -> projection 32 -> proj_width (GELU) -> 2 output channels (Re, Im of the
// scattered density). Kept modes: ky = 0 .. modes-1 of the half spectrum and
// kx = 0 .. modes-1, G-modes .. G-1 of the full one, i.e. the two corner
// blocks of the standard FNO.
//
// Activations are channel-last, [batch][x][y][channel] in FP32; the spectral
// transforms are truncated DFTs (only the kept modes are ever formed), done
// as three passes: along y (real <-> half spectrum), along x (complex), and
// the per-mode 32 x 32 complex channel mixing.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace lsg {

constexpr int kFnoWidth = 32;    // hidden channels (one per lane)
constexpr int kFnoIn = 6;        // input channels
constexpr int kFnoOut = 2;       // output channels
constexpr int kFnoMaxBatch = 64; // samples per forward / training step

struct FnoShape {
  int grid = 128;       // G: samples per axis (power of two, <= 256)
  int modes = 24;       // M: kept modes per axis (2 M <= G, M <= 32)
  int layers = 4;       // Fourier layers
  int proj = 128;       // hidden width of the projection (<= 128, multiple of 32)
};

// Offsets of the parameter groups in the flat FP32 parameter vector.
struct FnoLayout {
  long long lift_w = 0, lift_b = 0;        // [32][6], [32]
  std::vector<long long> spec, pw_w, pw_b; // per layer: [2M][M][32][32] complex, [32][32], [32]
  long long p1_w = 0, p1_b = 0;            // [proj][32], [proj]
  long long p2_w = 0, p2_b = 0;            // [2][proj], [2]
  long long total = 0;
  void build(const FnoShape& s);
};

struct FnoNet {
  int device = 0;
  FnoShape shape;
  FnoLayout lay;
  float* params = nullptr;
  float* grads = nullptr;
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  int adam_t = 0;
  float2* tw = nullptr;  // cos/sin(2 pi k / G), k < G
  // Activations and gradients for up to `cap` samples; `generation` counts
  // their reallocations (a captured launch sequence is valid for one).
  int cap = 0;
  unsigned long long generation = 0;
  std::vector<float*> h;  // layers + 1 inputs/outputs of the Fourier layers, [P][32]
  std::vector<float*> z;  // pre-activations, [P][32]
  std::vector<float2*> H2;// spectral inputs of each layer, [B][2M*M][32]
  float2 *H1 = nullptr, *O = nullptr, *G1 = nullptr;  // [B][G][M][32], [B][2M*M][32], [B][G][M][32]
  float *u = nullptr;     // projection pre-activation [P][proj]
  float *out = nullptr;   // [P][2]
  float *dout = nullptr, *dz = nullptr, *dh0 = nullptr, *dh1 = nullptr, *du = nullptr;
  float *sums = nullptr;  // per-sample |t|^2, |o - t|^2
  float *loss = nullptr;  // mean relative squared error of the last loss_grad
  int launches = 0;       // kernels launched by the last forward

  bool init(int dev, const FnoShape& s, unsigned long long seed, std::string& err);
  void release();
  cudaError_t ensure(int batch);
  // out[b][x][y][2] = net(in[b][x][y][6]). ssq (device, one float per sample,
  // may be null): the field channels are divided by sqrt(ssq/G^2) on input
  // and the outputs multiplied by it, which makes the net's linear use scale
  // invariant (the preconditioner's case). A single sample runs as one
  // cooperative launch (forward1) where the device allows it.
  cudaError_t forward(int batch, const float* in, float* out, const float* ssq, cudaStream_t s);
  // The layer-by-layer kernels (the training forward: keeps z and u).
  cudaError_t forward_layers(int batch, const float* in, float* out, const float* ssq, cudaStream_t s);
  cudaError_t forward1(const float* in, float* out, const float* ssq, cudaStream_t s);
  bool fused_ok();
  int fused = 0;         // 0: not checked, 1: forward1 available, -1: not available
  int fused_blocks = 0;  // co-resident blocks of forward1
  // Forward, loss = mean_b |o_b - t_b|^2 / |t_b|^2 (device scalar), backward
  // into grads (overwritten).
  cudaError_t loss_grad(int batch, const float* in, const float* target, cudaStream_t s);
  cudaError_t adam(float lr, float beta1, float beta2, float eps, cudaStream_t s);
};

// Training batches from superpositions of solved fields (fno.cu):
// for sample b with scatterer s = sidx[b] < S and coefficients c = coef[b][:nb],
//   f = sum_m c_m F[s][m],  t = sum_m c_m PHI[s][m]   (complex grid fields)
// scaled so that f has unit RMS, then in[b] = (q_s, Re f, Im f, kap[s], x, y)
// and target[b] = (Re t, Im t). An index outside [0, S) gives a zero sample.
cudaError_t fno_make_batch(int G, int batch, int nb, int S, const float2* F, const float2* PHI, const float* Q,
                           const float* kap, const int* sidx, const float2* coef, float* in, float* target,
                           float* ssq, cudaStream_t s);

}  // namespace lsg

// MLP inverse-CDF surrogate for the thermal scattering sampler: parameter
// layout, device buffers and the host-side entry points (mc_mlp.cu).
//
// Each network maps 16 input features (a few used, the rest zero) through
// three hidden layers of width 128 (SiLU) to one output:
//     x[16] -> 128 -> 128 -> 128 -> 1
// Hidden-layer products run on the tensor cores (tcgen05, FP32 accumulation
// in tensor memory): the forward products (training and sampling) take FP16
// operands -- 11 significant bits, which the surrogate's output precision
// needs -- and the backward products BF16 ones (range for the gradients);
// master weights and Adam moments are FP32.  The beta network predicts the quantile position of beta in
// [-E/kT, beta_cutoff]; the alpha network, given beta, the position of alpha
// between the kinematic bounds alpha_min(beta) and alpha_max(beta).
#pragma once

#include "mc_device.cuh"

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cstdint>

namespace mcd {

constexpr int kMlpWidth = 128;
constexpr int kMlpIn = 16;

// FP32 parameter vector of one network
constexpr int kMlpW1 = 0;                                  // [128][16]
constexpr int kMlpB1 = kMlpW1 + kMlpWidth * kMlpIn;        // [128]
constexpr int kMlpW2 = kMlpB1 + kMlpWidth;                 // [128][128]
constexpr int kMlpB2 = kMlpW2 + kMlpWidth * kMlpWidth;
constexpr int kMlpW3 = kMlpB2 + kMlpWidth;
constexpr int kMlpB3 = kMlpW3 + kMlpWidth * kMlpWidth;
constexpr int kMlpW4 = kMlpB3 + kMlpWidth;                 // [128]
constexpr int kMlpB4 = kMlpW4 + kMlpWidth;                 // [1]
constexpr int kMlpParams = kMlpB4 + 1;

// trained box and input scaling shared by training and inference
struct MlpBox {
  double logE0, logE1;   // ln E range
  double T0, T1;         // temperature range (K)
  double beta_cutoff;
  double awr;
  double beta_scale;     // ln(1 + |beta|) normalisation of the alpha network's beta input
};

// one network's device state
struct MlpNet {
  float* p = nullptr;       // [kMlpParams] master weights
  float* g = nullptr;       // gradients
  float* m = nullptr;       // Adam moments
  float* v = nullptr;
  __half* W1 = nullptr;          // [128][16] forward copies (FP16)
  __half* W2 = nullptr;          // [128][128]
  __half* W3 = nullptr;
  __nv_bfloat16* W2t = nullptr;  // BF16 transposes for the backward products
  __nv_bfloat16* W3t = nullptr;
};

// scratch of one training step over a batch of B samples
struct MlpBatch {
  int B = 0;
  __half* X = nullptr;           // [B][16] forward input
  __nv_bfloat16* Xt = nullptr;   // [16][B]
  float* y = nullptr;            // [B] targets
  float* Z1 = nullptr;           // [B][128] pre-activations
  float* Z2 = nullptr;
  float* Z3 = nullptr;
  __half* H1 = nullptr;          // [B][128] forward activations
  __half* H2 = nullptr;
  __nv_bfloat16* H1t = nullptr;  // [128][B] BF16 copies for the weight gradients
  __nv_bfloat16* H2t = nullptr;
  __nv_bfloat16* dZ3 = nullptr;  // [B][128]
  __nv_bfloat16* dZ2 = nullptr;
  __nv_bfloat16* dZ3t = nullptr; // [128][B]
  __nv_bfloat16* dZ2t = nullptr;
  __nv_bfloat16* dZ1t = nullptr;
  float* loss = nullptr;         // [1] sum of squared errors (with a StepState: [steps], one per step)
};

// A training step whose step-dependent values live on the device, so that
// one captured CUDA graph replays every step: `step` (1-based) selects the
// step's batch, its slot of the loss array and its row of `sched`
// (learning rate and Adam's two bias corrections); the weight refresh at the
// end of the step advances it.
struct StepState {
  int* step = nullptr;
  const float* sched = nullptr;  // [steps][3]: lr, 1 / (1 - 0.9^t), 1 / (1 - 0.999^t)
};

// launches (mc_mlp.cu); all stream-ordered
cudaError_t mlp_refresh_weights(const MlpNet& net, cudaStream_t s, int* advance_step = nullptr);
// with st.step set, b.loss is the per-step loss array (zeroed by the caller)
cudaError_t mlp_forward_backward(const MlpNet& net, const MlpBatch& b, cudaStream_t s, const StepState& st = {});
cudaError_t mlp_adam(const MlpNet& net, int step, float lr, cudaStream_t s);
cudaError_t mlp_adam(const MlpNet& net, const StepState& st, cudaStream_t s);
// inference on a batch of inputs (debug/grad-check path): out[B]
cudaError_t mlp_forward(const MlpNet& net, const MlpBatch& b, float* out, cudaStream_t s);

// surrogate sampler: beta then alpha for (E[i], T[i]) with Philox streams;
// samples outside the trained box fall back to the FP32 POD sampler
cudaError_t launch_sample_tsl_mlp(const DevTSL* tsl, const MlpNet& beta_net, const MlpNet& alpha_net,
                                  const MlpBox& box, const double* E, const double* T, unsigned long long n,
                                  unsigned long long key, double* beta, double* alpha, unsigned long long* failures,
                                  int num_sms, cudaStream_t s);

// the same networks on the thermal-scatter queue: rows (E, T, u1, u2) of
// parked particles, *count of them (at most cap, read on the device), to
// (beta, alpha) in FP32
cudaError_t launch_sample_tsl_mlp_queue(const MlpNet& beta_net, const MlpNet& alpha_net, const MlpBox& box,
                                        const float4* qin, const unsigned long long* count, unsigned long long cap,
                                        float2* qout, int num_sms, cudaStream_t s);

// training data: inputs and quantile targets from POD samples
cudaError_t launch_mlp_features_beta(const MlpBox& box, const double* E, const double* T, const double* u,
                                     const double* beta, unsigned long long n, __half* X, float* y,
                                     cudaStream_t s);
cudaError_t launch_mlp_features_alpha(const MlpBox& box, const double* E, const double* T, const double* beta,
                                      const double* u, const double* alpha, unsigned long long n, __half* X,
                                      float* y, cudaStream_t s);
// dst[i] = src[i / K] for i < n; u[i] = ((i mod K) + 1/2) / K
cudaError_t launch_expand(const double* src, unsigned long long n, int K, double* dst, cudaStream_t s);
cudaError_t launch_quantile_u(double* u, unsigned long long n, int K, cudaStream_t s);
// the device flag a timed-out tensor-core wait sets
int* mlp_error_flag();

// Guided sampler: the guide network (same layout as the surrogate networks:
// 16 inputs, three hidden layers of 128, one output) predicts where
// SampleAlpha's CDF bisection ends for each kinematic bound; the POD
// sampler then confirms or walks from there, so the samples are exactly the
// FP32 POD sampler's for the same random numbers.
// training rows: 2 per sample (the two bounds), n samples
cudaError_t launch_guide_data(const DevTSL* tsl, const MlpBox& box, unsigned long long key, unsigned long long n,
                              __half* X, float* y, unsigned long long* failures, cudaStream_t s);
// array form: Philox stream of row i keyed by (key, i), as the POD sampler's;
// `fast` selects the POD form reproduced (FP32 or exact FP64)
cudaError_t launch_sample_tsl_guided(const DevTSL* tsl, const MlpNet& guide, const MlpBox& box, bool fast,
                                     const double* E, const double* T, unsigned long long n, unsigned long long key,
                                     double* beta, double* alpha, unsigned long long* failures, int num_sms,
                                     cudaStream_t s);
// queue form: parked rows, *count of them (at most cap, read on the device);
// fast: the FP32 POD form, else the exact (FP64) one
cudaError_t launch_sample_tsl_guided_queue(const DevTSL* tsl, const MlpNet& guide, const MlpBox& box, bool fast,
                                           const GuideRow* rows, const unsigned long long* count,
                                           unsigned long long cap, unsigned long long run_key, GuideOut* out,
                                           int num_sms, cudaStream_t s);
// the POD sampler over the same queue, bisection without the network
cudaError_t launch_sample_tsl_pod_queue(const DevTSL* tsl, bool fast, const GuideRow* rows,
                                        const unsigned long long* count, unsigned long long cap,
                                        unsigned long long run_key, GuideOut* out, int num_sms, cudaStream_t s);
// per-condition sort of K samples (K a power of two <= 1024) in place
cudaError_t launch_segment_sort(double* v, unsigned long long n_segments, int K, cudaStream_t s);
// gathers a random batch (Philox key, step) of B rows of X / y into the
// batch buffers (and X transposed)
cudaError_t launch_mlp_gather(const __half* X, const float* y, unsigned long long n, unsigned long long key,
                              int step, const MlpBatch& b, cudaStream_t s, const int* step_ptr = nullptr);
// sampler-side POD draws used to build the training sets
cudaError_t launch_tsl_beta_draws(const DevTSL* tsl, const double* E, const double* T, unsigned long long n,
                                  unsigned long long key, double* beta, unsigned long long* failures, cudaStream_t s);
cudaError_t launch_tsl_alpha_draws(const DevTSL* tsl, const double* E, const double* T, const double* beta,
                                   unsigned long long n, unsigned long long key, double* alpha,
                                   unsigned long long* failures, cudaStream_t s);

}  // namespace mcd

// Thermal scattering sampler and cross-section kernels (one query per
// thread) behind mc_sample_tsl / mc_tsl_total: ThermalScattering::SampleBeta
// then SampleAlpha for given (E, T) pairs, as ThermalScattering::Scatter
// draws them (src/ThermalScattering.cpp:159-171).
#include "mc_kernels.cuh"
#include "mc_tsl.cuh"

namespace mcd {

namespace {

template <bool FAST, class Rng>
__global__ void __launch_bounds__(256) k_sample_tsl(const DevTSL* tsl, const double* E, const double* T,
                                                    unsigned long long n, unsigned long long seed,
                                                    unsigned long long key, double* beta, double* alpha,
                                                    unsigned long long* failures) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  bool failed = false;
  if (i < n) {
    const DevTSL& t = *tsl;
    Rng rng;
    if constexpr (std::is_same_v<Rng, MinstdRng>) rng.seed(seed + i);
    else rng.init(key, i, 2);
    const double e = E[i], temp = T[i];
    double b = CUDART_NAN, a = CUDART_NAN;
    if (tsl_sample_beta<FAST>(t, rng, e, temp, b)) {
      if (!tsl_sample_alpha<FAST>(t, rng, b, e, temp, a)) {
        a = CUDART_NAN;
        failed = true;
      }
    }
    else {
      b = CUDART_NAN;
      failed = true;
    }
    beta[i] = b;
    alpha[i] = a;
  }
  const unsigned mask = __ballot_sync(0xffffffffu, failed);
  if (mask && (threadIdx.x & 31) == static_cast<unsigned>(__ffs(mask) - 1))
    atomicAdd(failures, static_cast<unsigned long long>(__popc(mask)));
}

__global__ void k_tsl_total(const DevTSL* tsl, const double* E, const double* T, unsigned long long n, double* out) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) out[i] = tsl_total(*tsl, E[i], T[i]);
}

}  // namespace

cudaError_t launch_sample_tsl(const DevTSL* tsl, bool fast, int rng_mode, const double* E, const double* T,
                              unsigned long long n, unsigned long long seed, unsigned long long key, double* beta,
                              double* alpha, unsigned long long* failures, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  const unsigned blocks = static_cast<unsigned>((n + 255) / 256);
  if (rng_mode == 1) {
    if (fast) k_sample_tsl<true, MinstdRng><<<blocks, 256, 0, stream>>>(tsl, E, T, n, seed, key, beta, alpha, failures);
    else k_sample_tsl<false, MinstdRng><<<blocks, 256, 0, stream>>>(tsl, E, T, n, seed, key, beta, alpha, failures);
  }
  else {
    if (fast) k_sample_tsl<true, PhiloxRng><<<blocks, 256, 0, stream>>>(tsl, E, T, n, seed, key, beta, alpha, failures);
    else k_sample_tsl<false, PhiloxRng><<<blocks, 256, 0, stream>>>(tsl, E, T, n, seed, key, beta, alpha, failures);
  }
  return cudaGetLastError();
}

cudaError_t launch_tsl_total(const DevTSL* tsl, const double* E, const double* T, unsigned long long n, double* out,
                             cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  k_tsl_total<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(tsl, E, T, n, out);
  return cudaGetLastError();
}

}  // namespace mcd

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

// ---------------------------------------------------------------------------
// multigroup transfer of thermal scatters

namespace {

// every row's (E, T) repeated over its n samples
__global__ void k_expand_rows(const double* E_rows, const double* T_rows, unsigned long long n,
                              unsigned long long total, double* E, double* T) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const unsigned long long r = i / n;
  E[i] = E_rows[r];
  T[i] = T_rows[r];
}

// outgoing group of each sample: E' = E + beta k T as
// ThermalScattering::Scatter forms it (src/ThermalScattering.cpp:166,
// (beta k) T, no contraction), in the group g with bounds[g + 1] <= E' <
// bounds[g] (bounds descending; above the first bound: group 0, below the
// last: group G - 1).  Failed samples (NaN beta) are not binned.  Grid:
// blocks.x over a row's samples, blocks.y over the rows.
__global__ void __launch_bounds__(256) k_group_bins(const double* beta, unsigned long long n, const double* E_rows,
                                                   const double* T_rows, const double* bounds, int G,
                                                   unsigned long long* counts) {
  __shared__ double b[kMaxTransferGroups + 1];
  __shared__ unsigned h[kMaxTransferGroups];
  const unsigned r = blockIdx.y;
  for (int i = threadIdx.x; i <= G; i += blockDim.x) b[i] = bounds[i];
  for (int i = threadIdx.x; i < G; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const double e = E_rows[r];
  const double T = T_rows[r];
  const double* x = beta + static_cast<unsigned long long>(r) * n;
  for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    const double bt = x[i];
    if (bt != bt) continue;
    const double ep = __dadd_rn(e, __dmul_rn(__dmul_rn(bt, kBoltzmann), T));
    int g = 0;
    while (g < G - 1 && ep < b[g + 1]) g++;
    atomicAdd(&h[g], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < G; i += blockDim.x)
    if (h[i]) atomicAdd(counts + static_cast<unsigned long long>(r) * G + i, static_cast<unsigned long long>(h[i]));
}

}  // namespace

cudaError_t launch_expand_rows(const double* E_rows, const double* T_rows, unsigned rows, unsigned long long n,
                               double* E, double* T, cudaStream_t stream) {
  const unsigned long long total = static_cast<unsigned long long>(rows) * n;
  if (total == 0) return cudaSuccess;
  k_expand_rows<<<static_cast<unsigned>((total + 255) / 256), 256, 0, stream>>>(E_rows, T_rows, n, total, E, T);
  return cudaGetLastError();
}

cudaError_t launch_group_bins(const double* beta, unsigned rows, unsigned long long n, const double* E_rows,
                              const double* T_rows, const double* bounds, int G, unsigned long long* counts,
                              cudaStream_t stream) {
  if (rows == 0 || n == 0) return cudaSuccess;
  if (G < 1 || G > kMaxTransferGroups || rows > 65535) return cudaErrorInvalidValue;
  const unsigned long long per = (n + 255) / 256;
  const dim3 grid(static_cast<unsigned>(per < 64 ? per : 64), rows);
  k_group_bins<<<grid, 256, 0, stream>>>(beta, n, E_rows, T_rows, bounds, G, counts);
  return cudaGetLastError();
}

}  // namespace mcd

// Thin SVD for the POD table pipeline, FP64, by one-sided Jacobi rotations
// (Hestenes, J. SIAM 6 (1958) 51-90).
//
// A (m x n, column-major, m >= n) is orthogonalised one column pair at a
// time: the rotation of columns (i, j) that makes them orthogonal is
// applied to A and accumulated in V (n x n, starting as the identity).
// When a whole sweep over the pairs finds every pair orthogonal to within
// the tolerance, A V = U diag(S): the column norms are the singular values
// and the normalised columns the left singular vectors.
//
// The pairs of a sweep follow the round-robin (circle) order: with the
// columns padded to an even count p, step s (0 .. p - 2) pairs position k
// with position p - 1 - k, where position 0 holds column 0 and position
// k >= 1 holds column 1 + (k - 1 + s) mod (p - 1).  The p / 2 pairs of a
// step are disjoint, so one CTA per pair rotates them in parallel, and over
// the p - 1 steps of a sweep every pair meets exactly once.
#include "mc_kernels.cuh"

namespace mcd {

namespace {

constexpr int kSvdThreads = 256;

__device__ __forceinline__ int circle_column(int k, int s, int p) { return k == 0 ? 0 : 1 + (k - 1 + s) % (p - 1); }

// sums of the CTA's three partial sums, returned to every thread
__device__ __forceinline__ void block_sum3(double& a, double& b, double& c, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    sh[warp * 3 + 0] = a;
    sh[warp * 3 + 1] = b;
    sh[warp * 3 + 2] = c;
  }
  __syncthreads();
  a = b = c = 0.0;
  for (int w = 0; w < kSvdThreads / 32; w++) {
    a += sh[w * 3 + 0];
    b += sh[w * 3 + 1];
    c += sh[w * 3 + 2];
  }
}

__global__ void __launch_bounds__(kSvdThreads) k_jacobi_step(double* A, double* V, int m, int n, int p, int s,
                                                             double tol, unsigned* rotations) {
  __shared__ double sh[3 * kSvdThreads / 32];
  int i = circle_column(blockIdx.x, s, p), j = circle_column(p - 1 - blockIdx.x, s, p);
  if (i > j) {
    const int t = i;
    i = j;
    j = t;
  }
  if (j >= n) return;  // paired with the padding column
  double* ai = A + static_cast<size_t>(i) * m;
  double* aj = A + static_cast<size_t>(j) * m;
  double alpha = 0.0, beta = 0.0, gamma = 0.0;
  for (int r = threadIdx.x; r < m; r += kSvdThreads) {
    const double x = ai[r], y = aj[r];
    alpha = fma(x, x, alpha);
    beta = fma(y, y, beta);
    gamma = fma(x, y, gamma);
  }
  block_sum3(alpha, beta, gamma, sh);
  // every thread holds the same sums, so all take the same branch
  if (gamma == 0.0 || fabs(gamma) <= tol * sqrt(alpha) * sqrt(beta)) return;
  // the smaller root t of t^2 + 2 zeta t - 1 = 0 (rotation angle below pi/4)
  const double zeta = (beta - alpha) / (2.0 * gamma);
  const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(fma(zeta, zeta, 1.0)));
  const double c = 1.0 / sqrt(fma(t, t, 1.0)), sn = c * t;
  for (int r = threadIdx.x; r < m; r += kSvdThreads) {
    const double x = ai[r], y = aj[r];
    ai[r] = c * x - sn * y;
    aj[r] = sn * x + c * y;
  }
  double* vi = V + static_cast<size_t>(i) * n;
  double* vj = V + static_cast<size_t>(j) * n;
  for (int r = threadIdx.x; r < n; r += kSvdThreads) {
    const double x = vi[r], y = vj[r];
    vi[r] = c * x - sn * y;
    vj[r] = sn * x + c * y;
  }
  if (threadIdx.x == 0) atomicAdd(rotations, 1u);
}

__global__ void __launch_bounds__(kSvdThreads) k_column_norms(const double* A, int m, double* S) {
  __shared__ double sh[3 * kSvdThreads / 32];
  const double* a = A + static_cast<size_t>(blockIdx.x) * m;
  double s2 = 0.0, u = 0.0, w = 0.0;
  for (int r = threadIdx.x; r < m; r += kSvdThreads) s2 = fma(a[r], a[r], s2);
  block_sum3(s2, u, w, sh);
  if (threadIdx.x == 0) S[blockIdx.x] = sqrt(s2);
}

__global__ void k_identity(double* V, int n) {
  const size_t k = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < static_cast<size_t>(n) * n) V[k] = (k / n == k % n) ? 1.0 : 0.0;
}

}  // namespace

cudaError_t launch_jacobi_init(double* V, int n, cudaStream_t stream) {
  const size_t nn = static_cast<size_t>(n) * n;
  k_identity<<<static_cast<unsigned>((nn + 255) / 256), 256, 0, stream>>>(V, n);
  return cudaGetLastError();
}

cudaError_t launch_jacobi_sweep(double* A, double* V, int m, int n, double tol, unsigned* rotations,
                                cudaStream_t stream) {
  const int p = n + (n & 1);
  for (int s = 0; s < p - 1; s++) {
    k_jacobi_step<<<p / 2, kSvdThreads, 0, stream>>>(A, V, m, n, p, s, tol, rotations);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_column_norms(const double* A, int m, int n, double* S, cudaStream_t stream) {
  k_column_norms<<<n, kSvdThreads, 0, stream>>>(A, m, S);
  return cudaGetLastError();
}

}  // namespace mcd

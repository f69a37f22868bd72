// MLP surrogate kernels (layout and interfaces in mc_mlp.cuh).
//
// Training products, per step over a batch of B samples (B a multiple of
// 128), all C = A * B^T with K-major BF16 operands on the tensor cores:
//   forward   Z1 = X W1^T, Z2 = H1 W2^T, Z3 = H2 W3^T      (M = B, N = 128)
//   backward  dH2 = dZ3 W3, dH1 = dZ2 W2                   (M = B, N = 128)
//             dW3 = dZ3^T H2, dW2 = dZ2^T H1, dW1 = dZ1^T X (M = 128, K = B,
//             split over K across CTAs, FP32 atomics)
// Epilogues fuse bias, SiLU and its derivative, the transposed copies the
// weight-gradient products read, and the bias-gradient column sums.  The
// output layer (128 -> 1) and the loss run on the CUDA cores.
#include "mc_mlp.cuh"
#include "mc_tc.cuh"
#include "mc_tsl.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <type_traits>

namespace mcd {

namespace {

using bf16 = __nv_bfloat16;
using f16 = __half;
constexpr long long kWaitCycles = 2000000000LL;  // ~1 s: an MMA never takes that long

// The activation is evaluated the same way in training and in the sampler,
// so that the trained function is the one the sampler runs:
//   hidden layers: packed FP16, silu(z) = h + h tanh(h) with h = z / 2, from
//     the hardware's packed tanh (one MUFU operation per pair) and a packed
//     fma -- the result is an FP16 activation either way;
//   output layer: FP32, h + h tanh(h) with the FP32 hardware tanh.
// Gradients use the derivative of the exact SiLU.
__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float silu_h(float h) { return fmaf(h, tanh_approx(h), h); }
__device__ __forceinline__ float silu_t(float z) { return silu_h(0.5f * z); }
__device__ __forceinline__ __half2 silu2_f16(float h0, float h1) {
  const __half2 h = __floats2half2_rn(h0, h1);
  __half2 t;
  asm("tanh.approx.f16x2 %0, %1;"
      : "=r"(*reinterpret_cast<uint32_t*>(&t))
      : "r"(*reinterpret_cast<const uint32_t*>(&h)));
  return __hfma2(h, t, h);
}
__device__ __forceinline__ float dsilu(float z) {
  const float s = __fdividef(1.0f, 1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// generic GEMM: one CTA (128 threads) computes rows [m0, m0 + 128) x columns
// [n0, n0 + NT) of C = A[M x K] * B[N x K]^T over the K range of its split
// (blockIdx.z, at most kGemmMaxK columns).  Thread 0 issues every operand
// copy of that range up front as TMA boxes of R rows x 8 columns (16 bytes
// a row), one mbarrier per kGemmStageK columns, then issues each stage's
// MMAs as soon as its copies have landed, so the second stage's copies
// overlap the first stage's products.  A box lands as R * 16 contiguous
// bytes, so the element (row, k) of the K range sits at byte
//     (k / 8) * R * 16 + row * 16 + (k % 8) * 2
// -- the canonical K-major layout without swizzling, core matrices (8 rows
// x 16 B) 128 B apart along the rows (SBO) and R * 16 B apart along K
// (LBO).  The accumulator lives in tensor memory; the epilogue reads it 32
// columns at a time, and each warp turns its 32 x 32 block around in shared
// memory (the operand tiles' space, free once the products are done) so
// that the epilogues' row-major stores, transposed stores and atomics all
// run along contiguous addresses.
constexpr int kGemmStageK = 64;
constexpr int kGemmMaxK = 128;
constexpr int kGemmMaxStages = kGemmMaxK / kGemmStageK;
constexpr int kStagePitch = 33;  // floats per row of a warp's 32 x 32 block (conflict-free both ways)
constexpr size_t kGemmEpiBytes = 4 * 32 * kStagePitch * sizeof(float);

struct GemmArgs {
  int k_split;  // K per CTA (a multiple of 16, at most kGemmMaxK)
  int* err;     // set when a copy or an MMA wait timed out
};

__host__ __device__ constexpr size_t gemm_smem_bytes(int NT, int k_split) {
  const size_t ops = static_cast<size_t>(128 + NT) * k_split * 2;
  return ops > kGemmEpiBytes ? ops : kGemmEpiBytes;
}

template <int NT, class Epi, bool F16>
__global__ void __launch_bounds__(128) k_gemm(const __grid_constant__ CUtensorMap tmA,
                                              const __grid_constant__ CUtensorMap tmB, const GemmArgs a,
                                              const Epi epi) {
  static_assert(NT % 16 == 0 && NT >= 16 && NT <= 128, "NT");
  constexpr int kCols = NT < 32 ? 32 : NT;  // tensor-memory columns (power of two >= 32)
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) unsigned long long full[kGemmMaxStages];
  __shared__ __align__(8) unsigned long long done;
  __shared__ uint32_t tmem_slot;
  __shared__ int issue_ok;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * 128, n0 = blockIdx.y * NT;
  const int k_begin = blockIdx.z * a.k_split;
  const int stages = (a.k_split + kGemmStageK - 1) / kGemmStageK;
  const uint32_t sA = tc::smem_addr(smem);
  const uint32_t sB = sA + 128u * static_cast<uint32_t>(a.k_split) * 2u;
  if (warp == 0) tc::tmem_alloc(tc::smem_addr(&tmem_slot), kCols);
  if (tid == 0) {
    for (int s = 0; s < stages; s++) tc::mbar_init(tc::smem_addr(&full[s]), 1);
    tc::mbar_init(tc::smem_addr(&done), 1);
    tc::prefetch_tmap(&tmA);
    tc::prefetch_tmap(&tmB);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  if (tid == 0) {
    constexpr uint32_t idesc = F16 ? tc::idesc_f16_f32(128, NT) : tc::idesc_bf16_f32(128, NT);
    for (int s = 0; s < stages; s++) {
      const int kw = min(kGemmStageK, a.k_split - s * kGemmStageK);
      const uint32_t fb = tc::smem_addr(&full[s]);
      tc::mbar_expect_tx(fb, static_cast<uint32_t>((128 + NT) * kw * 2));
      for (int k = s * kGemmStageK; k < s * kGemmStageK + kw; k += 8) {
        tc::tma_load_2d(sA + static_cast<uint32_t>(k / 8) * 128u * 16u, &tmA, fb, k_begin + k, m0);
        tc::tma_load_2d(sB + static_cast<uint32_t>(k / 8) * NT * 16u, &tmB, fb, k_begin + k, n0);
      }
    }
    int landed = 0;
    for (; landed < stages; landed++) {
      if (!tc::mbar_wait(tc::smem_addr(&full[landed]), 0, kWaitCycles)) break;
      tc::fence_after_sync();
      const int kw = min(kGemmStageK, a.k_split - landed * kGemmStageK);
      for (int k = landed * kGemmStageK; k < landed * kGemmStageK + kw; k += 16) {
        const uint64_t ad = tc::smem_desc(sA + static_cast<uint32_t>(k / 8) * 128u * 16u, 128u * 16u, 128u);
        const uint64_t bd = tc::smem_desc(sB + static_cast<uint32_t>(k / 8) * NT * 16u, NT * 16u, 128u);
        tc::mma_bf16(tmem, ad, bd, idesc, k > 0 ? 1u : 0u);
      }
    }
    tc::mma_commit(tc::smem_addr(&done));
    issue_ok = landed == stages;
    // copies still in flight after a timed-out wait finish before the CTA
    // leaves (bounded again)
    for (int s = landed; s < stages; s++) tc::mbar_wait(tc::smem_addr(&full[s]), 0, kWaitCycles);
  }
  // the verdict is taken by the whole CTA so that every thread takes the
  // same branch
  const int fine = __syncthreads_and(tc::mbar_wait(tc::smem_addr(&done), 0, kWaitCycles) ? 1 : 0);
  tc::fence_after_sync();
  if (!fine || !issue_ok) {
    if (tid == 0) {
      atomicExch(a.err, 1);
      if (!fine) tc::mbar_wait(tc::smem_addr(&done), 0, kWaitCycles);  // the MMAs in flight, bounded again
    }
  }
  else {
    // epilogue: warp w owns tensor-memory lanes (rows) 32 w .. 32 w + 31
    float* st = reinterpret_cast<float*>(smem) + warp * 32 * kStagePitch;
    const int row0 = m0 + warp * 32;
#pragma unroll 1
    for (int c = 0; c < (NT + 31) / 32; c++) {
      float v[32];
      tc::tmem_ld32(tmem + (static_cast<uint32_t>(warp * 32) << 16) + c * 32, v);
#pragma unroll
      for (int j = 0; j < 32; j++) st[lane * kStagePitch + j] = v[j];
      __syncwarp();
      epi(row0, n0 + c * 32, st, NT - c * 32 < 32 ? NT - c * 32 : 32, lane);
      __syncwarp();
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kCols);
  }
}

// The epilogues see one warp's 32 x 32 block of the accumulator in shared
// memory: st[i * kStagePitch + j] = acc(row0 + i, col0 + j), j < ncol.

// z = acc + bias; keeps Z (FP32) and optionally H = SiLU(z) (FP16, the next
// forward operand) and H^T (BF16, for the weight gradients)
struct EpiForward {
  const float* bias;
  float* Z;
  f16* H;
  bf16* Ht;
  int B;
  __device__ __forceinline__ void operator()(int row0, int col0, float* st, int, int lane) const {
    // lanes 0-15 take column pairs of row i, lanes 16-31 those of row i + 1
    const int cp = 2 * (lane & 15), half = lane >> 4;
    const float b0 = bias[col0 + cp], b1 = bias[col0 + cp + 1];
#pragma unroll 4
    for (int i = 0; i < 32; i += 2) {
      const int r = i + half;
      float* e = st + r * kStagePitch + cp;
      const float z0 = e[0] + b0, z1 = e[1] + b1;
      const size_t o = static_cast<size_t>(row0 + r) * kMlpWidth + col0 + cp;
      *reinterpret_cast<float2*>(Z + o) = make_float2(z0, z1);
      if (H) {
        const __half2 h = silu2_f16(0.5f * z0, 0.5f * z1);
        *reinterpret_cast<__half2*>(H + o) = h;
        e[0] = __low2float(h);
        e[1] = __high2float(h);
      }
    }
    if (Ht) {
      __syncwarp();
#pragma unroll 4
      for (int j = 0; j < 32; j++)
        Ht[static_cast<size_t>(col0 + j) * B + row0 + lane] = __float2bfloat16_rn(st[lane * kStagePitch + j]);
    }
  }
};

// dz = acc * SiLU'(Zp); stores dZ (optional) and dZ^T, adds the column sums
// to the bias gradient
struct EpiBackward {
  const float* Zp;
  bf16* dZ;
  bf16* dZt;
  float* db;
  int B;
  __device__ __forceinline__ void operator()(int row0, int col0, float* st, int, int lane) const {
    // lane = column: Zp and dZ along rows, the column sum in a register;
    // the block's 32 Zp loads are all issued before the first is used
    float zp[32];
#pragma unroll
    for (int i = 0; i < 32; i++) zp[i] = Zp[static_cast<size_t>(row0 + i) * kMlpWidth + col0 + lane];
    float sum = 0.0f;
#pragma unroll
    for (int i = 0; i < 32; i++) {
      const float dz = st[i * kStagePitch + lane] * dsilu(zp[i]);
      if (dZ) dZ[static_cast<size_t>(row0 + i) * kMlpWidth + col0 + lane] = __float2bfloat16_rn(dz);
      st[i * kStagePitch + lane] = dz;
      sum += dz;
    }
    atomicAdd(db + col0 + lane, sum);
    __syncwarp();
    // lane = row: dZ^T along rows
#pragma unroll 4
    for (int j = 0; j < 32; j++)
      dZt[static_cast<size_t>(col0 + j) * B + row0 + lane] = __float2bfloat16_rn(st[lane * kStagePitch + j]);
  }
};

// C[row][col] += acc (split-K weight gradients); lane = column, so a warp's
// atomics of one row share cache lines
struct EpiAtomic {
  float* C;
  int ldc;
  __device__ __forceinline__ void operator()(int row0, int col0, float* st, int ncol, int lane) const {
    if (lane >= ncol) return;
#pragma unroll 4
    for (int i = 0; i < 32; i++)
      atomicAdd(C + static_cast<size_t>(row0 + i) * ldc + col0 + lane, st[i * kStagePitch + lane]);
  }
};

// cuTensorMapEncodeTiled from the driver, found through the runtime (no
// link against the driver library)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return static_cast<PFN_cuTensorMapEncodeTiled_v12000>(nullptr);
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

// tensor map of a row-major [rows x K] 16-bit operand (row pitch ld
// elements) whose boxes are `box_rows` rows x 8 columns
bool operand_map(CUtensorMap* m, const void* base, int ld, int rows, int K, int box_rows) {
  const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {static_cast<cuuint64_t>(K), static_cast<cuuint64_t>(rows)};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld) * 2};
  const cuuint32_t box[2] = {8, static_cast<cuuint32_t>(box_rows)};
  const cuuint32_t step[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<void*>(base), dims, strides, box, step,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// C = A[M x K] B[N x K]^T in tiles of 128 x NT, K split over `splits` CTAs
template <int NT, class Epi, class T>
cudaError_t gemm(const T* A, int lda, const T* B, int ldb, int M, int N, int K, int splits, int* err, const Epi& epi,
                 cudaStream_t s) {
  static_assert(sizeof(T) == 2, "16-bit operands");
  constexpr bool kF16 = std::is_same_v<T, f16>;
  if (M % 128 || N % NT || splits < 1 || K % splits) return cudaErrorInvalidValue;
  const int k_split = K / splits;
  if (k_split % 16 || k_split > kGemmMaxK || K > lda || K > ldb) return cudaErrorInvalidValue;
  if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15 || (lda | ldb) & 7)
    return cudaErrorInvalidValue;
  CUtensorMap ta, tb;
  if (!operand_map(&ta, A, lda, M, K, 128) || !operand_map(&tb, B, ldb, N, K, NT)) return cudaErrorInvalidValue;
  auto* kern = &k_gemm<NT, Epi, kF16>;
  const size_t smem = gemm_smem_bytes(NT, k_split);
  // the shared-memory limit is a per-device attribute: set once per device
  // (so that a captured training step makes no attribute call)
  static std::atomic<uint32_t> set_on{0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint32_t bit = dev < 32 ? 1u << dev : 0u;
  if (!bit || !(set_on.load() & bit)) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(gemm_smem_bytes(NT, kGemmMaxK)));
    if (e != cudaSuccess) return e;
    set_on.fetch_or(bit);
  }
  kern<<<dim3(M / 128, N / NT, splits), 128, smem, s>>>(ta, tb, GemmArgs{k_split, err}, epi);
  return cudaGetLastError();
}

// output layer, loss and the first backward step, one sample per thread:
// out = b4 + w4 . SiLU(Z3); e = out - y; dZ3 = (2e / B) w4 SiLU'(Z3)
// One CTA per 32 rows, one thread per column (128): the Z3 rows are read
// and dZ3's written along the rows (coalesced); a row's output is the sum
// of its four warps' partial sums; each thread keeps its column's dW4 and
// db3 sums over the 32 rows in registers (one atomic pair per column per
// CTA) and writes its column of dZ3^T for the 32 rows as four 16-byte
// stores.
constexpr int kHeadRows = 32;
__global__ void __launch_bounds__(128) k_head(const float* Z3, const float* p, const float* y, int B, bf16* dZ3,
                                              bf16* dZ3t, float* g, float* loss, const int* step) {
  __shared__ float part[4][kHeadRows];
  __shared__ float go_s[kHeadRows];
  if (step) loss += *step - 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = threadIdx.x;  // column
  const int row0 = blockIdx.x * kHeadRows;
  const float w4 = p[kMlpW4 + c];
  float z[kHeadRows];
#pragma unroll
  for (int i = 0; i < kHeadRows; i++) z[i] = Z3[static_cast<size_t>(row0 + i) * kMlpWidth + c];
#pragma unroll
  for (int i = 0; i < kHeadRows; i++) {
    const float s = warp_sum(silu_t(z[i]) * w4);
    if (lane == 0) part[warp][i] = s;
  }
  __syncthreads();
  if (warp == 0) {
    const int i = lane;
    const float out = p[kMlpB4] + part[0][i] + part[1][i] + part[2][i] + part[3][i];
    const float e = out - y[row0 + i];
    const float go = 2.0f * e / static_cast<float>(B);
    go_s[i] = go;
    const float se = warp_sum(e * e);
    const float sg = warp_sum(go);
    if (lane == 0) {
      atomicAdd(loss, se);
      atomicAdd(g + kMlpB4, sg);
    }
  }
  __syncthreads();
  float dw4 = 0.0f, db3 = 0.0f;
  uint32_t col[kHeadRows / 2];  // this column's dZ for the 32 rows, BF16 pairs
#pragma unroll
  for (int i = 0; i < kHeadRows; i += 2) {
    const float g0 = go_s[i], g1 = go_s[i + 1];
    const float dz0 = g0 * w4 * dsilu(z[i]);
    const float dz1 = g1 * w4 * dsilu(z[i + 1]);
    const bf16 h0 = __float2bfloat16_rn(dz0), h1 = __float2bfloat16_rn(dz1);
    dZ3[static_cast<size_t>(row0 + i) * kMlpWidth + c] = h0;
    dZ3[static_cast<size_t>(row0 + i + 1) * kMlpWidth + c] = h1;
    dw4 += g0 * silu_t(z[i]);
    dw4 += g1 * silu_t(z[i + 1]);
    db3 += dz0;
    db3 += dz1;
    col[i / 2] = static_cast<uint32_t>(__bfloat16_as_ushort(h0)) | (static_cast<uint32_t>(__bfloat16_as_ushort(h1)) << 16);
  }
  // rows row0 .. row0 + 31 of column c: 64 contiguous bytes (B and row0
  // are multiples of 32, so the address is 64-byte aligned)
  uint4* dst = reinterpret_cast<uint4*>(dZ3t + static_cast<size_t>(c) * B + row0);
#pragma unroll
  for (int k = 0; k < 4; k++) dst[k] = make_uint4(col[4 * k], col[4 * k + 1], col[4 * k + 2], col[4 * k + 3]);
  atomicAdd(g + kMlpW4 + c, dw4);
  atomicAdd(g + kMlpB3 + c, db3);
}

// forward output only
__global__ void k_head_forward(const float* Z3, const float* p, int B, float* out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= B) return;
  const float* z = Z3 + static_cast<size_t>(r) * kMlpWidth;
  float o = p[kMlpB4];
  for (int j = 0; j < kMlpWidth; j++) o = fmaf(silu_t(z[j]), p[kMlpW4 + j], o);
  out[r] = o;
}

// Adam (Kingma and Ba), bias-corrected
__global__ void k_adam(float* p, const float* g, float* m, float* v, int n, float lr, float c1, float c2,
                       const float* sched, const int* step) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (step) {
    const float* row = sched + 3 * (*step - 1);
    lr = row[0];
    c1 = row[1];
    c2 = row[2];
  }
  const float gi = g[i];
  const float mi = 0.9f * m[i] + 0.1f * gi;
  const float vi = 0.999f * v[i] + 0.001f * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + 1e-8f);
}

// FP16 forward weight copies and BF16 transposes from the FP32 master weights
__global__ void k_refresh(const float* p, f16* W1, f16* W2, f16* W3, bf16* W2t, bf16* W3t, int* advance_step) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  // the last launch of a step: the next step's counter (nothing here reads it)
  if (advance_step && i == 0) *advance_step += 1;
  if (i < kMlpWidth * kMlpIn) W1[i] = __float2half_rn(p[kMlpW1 + i]);
  if (i < kMlpWidth * kMlpWidth) {
    const int r = i / kMlpWidth, c = i % kMlpWidth;
    W2[i] = __float2half_rn(p[kMlpW2 + i]);
    W3[i] = __float2half_rn(p[kMlpW3 + i]);
    W2t[c * kMlpWidth + r] = __float2bfloat16_rn(p[kMlpW2 + i]);
    W3t[c * kMlpWidth + r] = __float2bfloat16_rn(p[kMlpW3 + i]);
  }
}

__device__ int g_mlp_err;

}  // namespace

cudaError_t mlp_refresh_weights(const MlpNet& net, cudaStream_t s, int* advance_step) {
  k_refresh<<<kMlpWidth * kMlpWidth / 256, 256, 0, s>>>(net.p, net.W1, net.W2, net.W3, net.W2t, net.W3t,
                                                          advance_step);
  return cudaGetLastError();
}

namespace {
int* mlp_err_ptr() {
  static int* p = nullptr;
  if (!p) cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_mlp_err);
  return p;
}
}  // namespace

cudaError_t mlp_forward(const MlpNet& net, const MlpBatch& b, float* out, cudaStream_t s) {
  int* err = mlp_err_ptr();
  cudaError_t e;
  if ((e = gemm<64>(b.X, kMlpIn, net.W1, kMlpIn, b.B, kMlpWidth, kMlpIn, 1, err,
                         EpiForward{net.p + kMlpB1, b.Z1, b.H1, nullptr, b.B}, s)) != cudaSuccess)
    return e;
  if ((e = gemm<64>(b.H1, kMlpWidth, net.W2, kMlpWidth, b.B, kMlpWidth, kMlpWidth, 1, err,
                         EpiForward{net.p + kMlpB2, b.Z2, b.H2, nullptr, b.B}, s)) != cudaSuccess)
    return e;
  if ((e = gemm<64>(b.H2, kMlpWidth, net.W3, kMlpWidth, b.B, kMlpWidth, kMlpWidth, 1, err,
                         EpiForward{net.p + kMlpB3, b.Z3, nullptr, nullptr, b.B}, s)) != cudaSuccess)
    return e;
  k_head_forward<<<(b.B + 127) / 128, 128, 0, s>>>(b.Z3, net.p, b.B, out);
  return cudaGetLastError();
}

cudaError_t mlp_forward_backward(const MlpNet& net, const MlpBatch& b, cudaStream_t s, const StepState& st) {
  int* err = mlp_err_ptr();
  const int B = b.B;
  // weight-gradient products split K = B into chunks of 128 samples
  const int splits = B / 128;
  cudaError_t e;
  if ((e = cudaMemsetAsync(net.g, 0, kMlpParams * sizeof(float), s)) != cudaSuccess) return e;
  if (!st.step && (e = cudaMemsetAsync(b.loss, 0, sizeof(float), s)) != cudaSuccess) return e;
  if ((e = gemm<64>(b.X, kMlpIn, net.W1, kMlpIn, B, kMlpWidth, kMlpIn, 1, err,
                         EpiForward{net.p + kMlpB1, b.Z1, b.H1, b.H1t, B}, s)) != cudaSuccess)
    return e;
  if ((e = gemm<64>(b.H1, kMlpWidth, net.W2, kMlpWidth, B, kMlpWidth, kMlpWidth, 1, err,
                         EpiForward{net.p + kMlpB2, b.Z2, b.H2, b.H2t, B}, s)) != cudaSuccess)
    return e;
  // Z3 only (H3 is recomputed from Z3 by the head)
  if ((e = gemm<64>(b.H2, kMlpWidth, net.W3, kMlpWidth, B, kMlpWidth, kMlpWidth, 1, err,
                         EpiForward{net.p + kMlpB3, b.Z3, nullptr, nullptr, B}, s)) != cudaSuccess)
    return e;
  k_head<<<B / kHeadRows, 128, 0, s>>>(b.Z3, net.p, b.y, B, b.dZ3, b.dZ3t, net.g, b.loss, st.step);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // layer 3: dW3 = dZ3^T H2; dH2 = dZ3 W3 -> dZ2
  if ((e = gemm<64>(b.dZ3t, B, b.H2t, B, kMlpWidth, kMlpWidth, B, splits, err, EpiAtomic{net.g + kMlpW3, kMlpWidth}, s)) !=
      cudaSuccess)
    return e;
  if ((e = gemm<64>(b.dZ3, kMlpWidth, net.W3t, kMlpWidth, B, kMlpWidth, kMlpWidth, 1, err,
                         EpiBackward{b.Z2, b.dZ2, b.dZ2t, net.g + kMlpB2, B}, s)) != cudaSuccess)
    return e;
  // layer 2: dW2 = dZ2^T H1; dH1 = dZ2 W2 -> dZ1 (transposed only)
  if ((e = gemm<64>(b.dZ2t, B, b.H1t, B, kMlpWidth, kMlpWidth, B, splits, err, EpiAtomic{net.g + kMlpW2, kMlpWidth}, s)) !=
      cudaSuccess)
    return e;
  if ((e = gemm<64>(b.dZ2, kMlpWidth, net.W2t, kMlpWidth, B, kMlpWidth, kMlpWidth, 1, err,
                         EpiBackward{b.Z1, nullptr, b.dZ1t, net.g + kMlpB1, B}, s)) != cudaSuccess)
    return e;
  // layer 1: dW1 = dZ1^T X
  return gemm<16>(b.dZ1t, B, b.Xt, B, kMlpWidth, kMlpIn, B, splits, err, EpiAtomic{net.g + kMlpW1, kMlpIn}, s);
}

cudaError_t mlp_adam(const MlpNet& net, int step, float lr, cudaStream_t s) {
  const float c1 = 1.0f / (1.0f - powf(0.9f, static_cast<float>(step)));
  const float c2 = 1.0f / (1.0f - powf(0.999f, static_cast<float>(step)));
  k_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(net.p, net.g, net.m, net.v, kMlpParams, lr, c1, c2, nullptr,
                                                  nullptr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return mlp_refresh_weights(net, s);
}

cudaError_t mlp_adam(const MlpNet& net, const StepState& st, cudaStream_t s) {
  k_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(net.p, net.g, net.m, net.v, kMlpParams, 0.0f, 0.0f, 0.0f, st.sched,
                                                  st.step);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return mlp_refresh_weights(net, s, st.step);
}

// ---------------------------------------------------------------------------
// features and targets (shared by training and inference)

namespace {

// The features feed BF16 operands and the networks' outputs carry BF16-level
// error, so everything around them runs in FP32 (the FP64 pipe is 1/64 of
// the FP32 rate on this part).  The same functions build the training
// inputs, so training and inference see identical features.
struct BoxF {
  float e_scale, e_shift;   // f0 = ln E * e_scale + e_shift  (maps [logE0, logE1] to [-1, 1])
  float t_scale, t_shift;   // f1 = T * t_scale + t_shift
  float beta_cutoff;
  float inv_beta_scale;
  float kB;                 // Boltzmann constant (MeV/K)
  float inv_awr;
  float r_scale, r_shift;   // f6 = ln(E / kT) * r_scale + r_shift (the box's range to [-1, 1])
};

__device__ __forceinline__ BoxF box_f(const MlpBox& b) {
  BoxF f;
  const double es = 2.0 / (b.logE1 - b.logE0), ts = 2.0 / (b.T1 - b.T0);
  f.e_scale = static_cast<float>(es);
  f.e_shift = static_cast<float>(-b.logE0 * es - 1.0);
  f.t_scale = static_cast<float>(ts);
  f.t_shift = static_cast<float>(-b.T0 * ts - 1.0);
  f.beta_cutoff = static_cast<float>(b.beta_cutoff);
  f.inv_beta_scale = static_cast<float>(1.0 / b.beta_scale);
  f.kB = static_cast<float>(kBoltzmann);
  f.inv_awr = static_cast<float>(1.0 / b.awr);
  const double r0 = b.logE0 - log(kBoltzmann * b.T1), r1 = b.logE1 - log(kBoltzmann * b.T0);
  const double rs = 2.0 / (r1 - r0);
  f.r_scale = static_cast<float>(rs);
  f.r_shift = static_cast<float>(-r0 * rs - 1.0);
  return f;
}

__device__ __forceinline__ float beta_min_of(const BoxF& b, float E, float T) { return -E / (b.kB * T); }

// features: ln E, T, u, logit(u) / 8, [alpha only: beta, beta's position],
// ln(E / kT) -- the free-gas scaling variable, on which the distributions
// mostly depend
__device__ __forceinline__ void base_features(const BoxF& b, float E, float T, float u, float* f) {
  const float lE = logf(E);
  f[0] = fmaf(lE, b.e_scale, b.e_shift);
  f[1] = fmaf(T, b.t_scale, b.t_shift);
  f[2] = fmaf(2.0f, u, -1.0f);
  f[3] = fminf(2.0f, fmaxf(-2.0f, (logf(u) - log1pf(-u)) * 0.125f));
  f[6] = fmaf(lE - logf(b.kB * T), b.r_scale, b.r_shift);
}

__device__ __forceinline__ void beta_features(const BoxF& b, float E, float T, float u, float (&f)[kMlpIn]) {
#pragma unroll
  for (int i = 0; i < kMlpIn; i++) f[i] = 0.0f;
  base_features(b, E, T, u, f);
}

__device__ __forceinline__ void alpha_features(const BoxF& b, float E, float T, float beta, float u,
                                               float (&f)[kMlpIn]) {
#pragma unroll
  for (int i = 0; i < kMlpIn; i++) f[i] = 0.0f;
  base_features(b, E, T, u, f);
  const float bmin = beta_min_of(b, E, T);
  f[4] = copysignf(log1pf(fabsf(beta)), beta) * b.inv_beta_scale;
  f[5] = 2.0f * (beta - bmin) / (b.beta_cutoff - bmin) - 1.0f;
}

// kinematic alpha bounds (sqrt E -+ sqrt E')^2 / (A kT) with E' = E + beta kT;
// sqrt E - sqrt E' is formed as -beta kT / (sqrt E + sqrt E') so that the
// lower bound keeps its relative accuracy as beta -> 0
__device__ __forceinline__ void alpha_range(const BoxF& b, float E, float T, float beta, float& lo, float& hi) {
  const float kT = b.kB * T;
  const float Ep = E + beta * kT;
  const float r = sqrtf(E), s = sqrtf(fmaxf(0.0f, Ep));
  const float d = Ep > 0.0f ? -beta * kT / (r + s) : r;
  const float inv = b.inv_awr / kT;
  lo = d * d * inv;
  hi = (r + s) * (r + s) * inv;
}

// The features enter the first product as FP16; each used feature k is
// split into its FP16 value (slot k) and the residual scaled by 2048 (slot
// 8 + k), so the product sees the FP32 feature to about 22 significant
// bits (one FP16 input would quantise E, T and the uniform to 2^-11).
constexpr int kMlpFeatures = 7;
constexpr float kResidualScale = 2048.0f;
__device__ __forceinline__ void split_features(const float (&f)[kMlpIn], f16 (&x)[kMlpIn]) {
#pragma unroll
  for (int i = 0; i < kMlpIn; i++) x[i] = __float2half_rn(0.0f);
#pragma unroll
  for (int k = 0; k < kMlpFeatures; k++) {
    const f16 hi = __float2half_rn(f[k]);
    x[k] = hi;
    x[8 + k] = __float2half_rn((f[k] - __half2float(hi)) * kResidualScale);
  }
}

__device__ __forceinline__ void store_features(const float (&f)[kMlpIn], f16* row) {
  f16 x[kMlpIn];
  split_features(f, x);
#pragma unroll
  for (int i = 0; i < kMlpIn; i++) row[i] = x[i];
}

// training targets: quantile positions of sorted samples within their
// condition (u = (k + 1/2) / K)
__global__ void k_features_beta(MlpBox box, const double* E, const double* T, const double* u, const double* beta,
                                unsigned long long n, f16* X, float* y) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const BoxF b = box_f(box);
  const float e = static_cast<float>(E[i]), t = static_cast<float>(T[i]);
  float f[kMlpIn];
  beta_features(b, e, t, static_cast<float>(u[i]), f);
  store_features(f, X + i * kMlpIn);
  const double bmin = beta_min_of(b, e, t);
  const double q = (beta[i] - bmin) / (box.beta_cutoff - bmin);
  y[i] = isfinite(q) ? static_cast<float>(q) : 0.5f;
}

__global__ void k_features_alpha(MlpBox box, const double* E, const double* T, const double* beta, const double* u,
                                 const double* alpha, unsigned long long n, f16* X, float* y) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const BoxF b = box_f(box);
  const float e = static_cast<float>(E[i]), t = static_cast<float>(T[i]), bt = static_cast<float>(beta[i]);
  float f[kMlpIn];
  alpha_features(b, e, t, bt, static_cast<float>(u[i]), f);
  store_features(f, X + i * kMlpIn);
  float lo, hi;
  alpha_range(b, e, t, bt, lo, hi);
  const double q = (alpha[i] - lo) / (static_cast<double>(hi) - lo);
  y[i] = isfinite(q) ? static_cast<float>(q) : 0.5f;
}

// bitonic sort of each K-value segment in shared memory (NaN last)
__global__ void __launch_bounds__(1024) k_segment_sort(double* v, int K) {
  __shared__ double s[1024];
  double* seg = v + static_cast<size_t>(blockIdx.x) * K;
  const int t = threadIdx.x;
  if (t < K) {
    const double x = seg[t];
    s[t] = x == x ? x : CUDART_INF;
  }
  __syncthreads();
  for (int size = 2; size <= K; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      if (t < K) {
        const int partner = t ^ stride;
        if (partner > t) {
          const bool up = (t & size) == 0;
          const double a = s[t], b = s[partner];
          if ((a > b) == up) {
            s[t] = b;
            s[partner] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  if (t < K) seg[t] = s[t];
}

// random batch: row r of the batch is sample philox(key, step, r) mod n
__global__ void k_gather(const f16* X, const float* y, unsigned long long n, unsigned long long key, int step,
                         const int* step_ptr, int B, f16* bX, bf16* bXt, float* by) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= B) return;
  if (step_ptr) step = *step_ptr;
  uint32_t c[4] = {static_cast<uint32_t>(r), static_cast<uint32_t>(step), 0x4D4C5000u, 0};
  philox4x32_10(c, static_cast<uint32_t>(key), static_cast<uint32_t>(key >> 32));
  const unsigned long long idx = ((static_cast<unsigned long long>(c[0]) << 32) | c[1]) % n;
#pragma unroll
  for (int f = 0; f < kMlpIn; f++) {
    const f16 v = X[idx * kMlpIn + f];
    bX[static_cast<size_t>(r) * kMlpIn + f] = v;
    bXt[static_cast<size_t>(f) * B + r] = __float2bfloat16_rn(__half2float(v));
  }
  by[r] = y[idx];
}

// POD draws for the training sets (exact form, Philox streams)
__global__ void k_beta_draws(const DevTSL* tsl, const double* E, const double* T, unsigned long long n,
                             unsigned long long key, double* beta, unsigned long long* failures) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  PhiloxRng rng;
  rng.init(key, i, 4);
  double b;
  if (!tsl_sample_beta<false>(*tsl, rng, E[i], T[i], b)) {
    b = CUDART_NAN;
    atomicAdd(failures, 1ull);
  }
  beta[i] = b;
}

__global__ void k_alpha_draws(const DevTSL* tsl, const double* E, const double* T, const double* beta,
                              unsigned long long n, unsigned long long key, double* alpha,
                              unsigned long long* failures) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  PhiloxRng rng;
  rng.init(key, i, 5);
  double a;
  if (!(beta[i] == beta[i]) || !tsl_sample_alpha<false>(*tsl, rng, beta[i], E[i], T[i], a)) {
    a = CUDART_NAN;
    atomicAdd(failures, 1ull);
  }
  alpha[i] = a;
}

unsigned blocks256(unsigned long long n) { return static_cast<unsigned>((n + 255) / 256); }

}  // namespace

namespace {
__global__ void k_expand(const double* src, unsigned long long n, int K, double* dst) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i / K];
}
__global__ void k_quantile_u(double* u, unsigned long long n, int K) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) u[i] = (static_cast<double>(i % K) + 0.5) / K;
}
}  // namespace

cudaError_t launch_expand(const double* src, unsigned long long n, int K, double* dst, cudaStream_t s) {
  k_expand<<<blocks256(n), 256, 0, s>>>(src, n, K, dst);
  return cudaGetLastError();
}

cudaError_t launch_quantile_u(double* u, unsigned long long n, int K, cudaStream_t s) {
  k_quantile_u<<<blocks256(n), 256, 0, s>>>(u, n, K);
  return cudaGetLastError();
}

cudaError_t launch_mlp_features_beta(const MlpBox& box, const double* E, const double* T, const double* u,
                                     const double* beta, unsigned long long n, __half* X, float* y,
                                     cudaStream_t s) {
  k_features_beta<<<blocks256(n), 256, 0, s>>>(box, E, T, u, beta, n, X, y);
  return cudaGetLastError();
}

cudaError_t launch_mlp_features_alpha(const MlpBox& box, const double* E, const double* T, const double* beta,
                                      const double* u, const double* alpha, unsigned long long n, __half* X,
                                      float* y, cudaStream_t s) {
  k_features_alpha<<<blocks256(n), 256, 0, s>>>(box, E, T, beta, u, alpha, n, X, y);
  return cudaGetLastError();
}

cudaError_t launch_segment_sort(double* v, unsigned long long n_segments, int K, cudaStream_t s) {
  if (K < 2 || K > 1024 || (K & (K - 1))) return cudaErrorInvalidValue;
  k_segment_sort<<<static_cast<unsigned>(n_segments), K, 0, s>>>(v, K);
  return cudaGetLastError();
}

cudaError_t launch_mlp_gather(const __half* X, const float* y, unsigned long long n, unsigned long long key,
                              int step, const MlpBatch& b, cudaStream_t s, const int* step_ptr) {
  k_gather<<<(b.B + 255) / 256, 256, 0, s>>>(X, y, n, key, step, step_ptr, b.B, b.X, b.Xt, b.y);
  return cudaGetLastError();
}

cudaError_t launch_tsl_beta_draws(const DevTSL* tsl, const double* E, const double* T, unsigned long long n,
                                  unsigned long long key, double* beta, unsigned long long* failures, cudaStream_t s) {
  k_beta_draws<<<blocks256(n), 256, 0, s>>>(tsl, E, T, n, key, beta, failures);
  return cudaGetLastError();
}

cudaError_t launch_tsl_alpha_draws(const DevTSL* tsl, const double* E, const double* T, const double* beta,
                                   unsigned long long n, unsigned long long key, double* alpha,
                                   unsigned long long* failures, cudaStream_t s) {
  k_alpha_draws<<<blocks256(n), 256, 0, s>>>(tsl, E, T, beta, n, key, alpha, failures);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// fused surrogate sampler: both networks' BF16 weights resident in shared
// memory; each of the CTA's two warpgroups works through its own 128-sample
// tiles (one sample per thread) with its own input and hidden tiles, its own
// 128 tensor-memory columns and its own mbarrier, so one warpgroup's
// epilogue overlaps the other's products.  Each layer is one tcgen05
// product into tensor memory followed by a per-row epilogue (bias, SiLU)
// that writes the next layer's operand tile.

namespace {

struct NetView {
  const float* p;
  const f16* W1;  // FP16 forward copies
  const f16* W2;
  const f16* W3;
};

constexpr int kGroups = 2;                                // warpgroups (tiles in flight) per CTA
constexpr uint32_t kTileW1 = kMlpWidth * kMlpIn * 2;      // 4 KB
constexpr uint32_t kTileW = kMlpWidth * kMlpWidth * 2;    // 32 KB
constexpr uint32_t kOffB1 = 0;                            // beta network W1
constexpr uint32_t kOffB2 = kOffB1 + kTileW1;
constexpr uint32_t kOffB3 = kOffB2 + kTileW;
constexpr uint32_t kOffA1 = kOffB3 + kTileW;              // alpha network
constexpr uint32_t kOffA2 = kOffA1 + kTileW1;
constexpr uint32_t kOffA3 = kOffA2 + kTileW;
constexpr uint32_t kOffG = kOffA3 + kTileW;               // per warpgroup: input tile, hidden tile
constexpr uint32_t kGroupBytes = kTileW1 + kTileW;
constexpr uint32_t kOffF = kOffG + kGroups * kGroupBytes; // FP32: per net b1 b2 b3 w4 (4 x 128) + b4
constexpr uint32_t kOffMisc = kOffF + 2 * (4 * kMlpWidth + 4) * 4;
constexpr uint32_t kSampleSmem = kOffMisc + 64;
static_assert(kSampleSmem <= 227 * 1024, "shared memory");

// warpgroup barrier (named barrier 1 + g, 128 threads) and its AND vote
__device__ __forceinline__ void wg_sync(int g) { asm volatile("bar.sync %0, 128;" ::"r"(1 + g) : "memory"); }
__device__ __forceinline__ bool wg_all(int g, bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.and.pred p, %2, 128, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(r)
      : "r"(v ? 1u : 0u), "r"(1 + g)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ void load_tile(uint8_t* dst, const f16* src, int K) {
  for (int c = threadIdx.x; c < kMlpWidth * (K / 8); c += blockDim.x) {
    const int row = c % kMlpWidth, kc = c / kMlpWidth;
    *reinterpret_cast<uint4*>(dst + tc::tile_offset(row, kc * 8, K)) =
        *reinterpret_cast<const uint4*>(src + static_cast<size_t>(row) * K + kc * 8);
  }
}

// one warpgroup's working set
struct Group {
  uint8_t* base;   // shared memory base
  uint32_t X, H;   // offsets of its input and hidden tiles
  uint32_t tmem;   // its 128 accumulator columns
  uint32_t mbar;
  uint32_t phase;
  int g, lt;       // warpgroup, thread within it (the tile row)
  bool ok;
};

// D = act_tile * W^T (K = 16 or 128)
__device__ __forceinline__ void layer_mma(Group& G, uint32_t act_off, uint32_t w_off, int K) {
  tc::fence_proxy_async();
  tc::fence_before_sync();
  wg_sync(G.g);
  if (G.lt == 0) {
    tc::fence_after_sync();
    const uint32_t a0 = tc::smem_addr(G.base + act_off), b0 = tc::smem_addr(G.base + w_off);
    constexpr uint32_t idesc = tc::idesc_f16_f32(128, kMlpWidth);
    for (int s = 0; s < K / 16; s++)
      tc::mma_bf16(G.tmem, tc::smem_desc(a0 + s * 256, 128, K * 16), tc::smem_desc(b0 + s * 256, 128, K * 16),
                   idesc, s > 0 ? 1u : 0u);
    tc::mma_commit(G.mbar);
  }
  if (!wg_all(G.g, tc::mbar_wait(G.mbar, G.phase, kWaitCycles))) G.ok = false;
  G.phase ^= 1;
  tc::fence_after_sync();
}

// h = SiLU(acc + bias) into the warpgroup's hidden tile (this thread's row);
// `hbias` holds bias / 2
__device__ __forceinline__ void hidden_epilogue(Group& G, const float* hbias) {
  const int w = G.lt >> 5;
  uint8_t* H = G.base + G.H;
#pragma unroll 1
  for (int c = 0; c < kMlpWidth / 32; c++) {
    float v[32];
    tc::tmem_ld32(G.tmem + (static_cast<uint32_t>(w * 32) << 16) + c * 32, v);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      __align__(16) __half2 h[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int k = q * 8 + 2 * j;
        h[j] = silu2_f16(fmaf(v[k], 0.5f, hbias[c * 32 + k]), fmaf(v[k + 1], 0.5f, hbias[c * 32 + k + 1]));
      }
      *reinterpret_cast<uint4*>(H + tc::tile_offset(G.lt, c * 32 + q * 8, kMlpWidth)) = *reinterpret_cast<uint4*>(h);
    }
  }
}

// b4 + w4 . SiLU(acc + b3); `f` holds b1/2, b2/2, b3/2, w4, b4
__device__ __forceinline__ float output_epilogue(Group& G, const float* f) {
  const int w = G.lt >> 5;
  const float* b3 = f + 2 * kMlpWidth;
  const float* w4 = f + 3 * kMlpWidth;
  float out = f[4 * kMlpWidth];
#pragma unroll 1
  for (int c = 0; c < kMlpWidth / 32; c++) {
    float v[32];
    tc::tmem_ld32(G.tmem + (static_cast<uint32_t>(w * 32) << 16) + c * 32, v);
#pragma unroll
    for (int j = 0; j < 32; j++) out = fmaf(silu_h(fmaf(v[j], 0.5f, b3[c * 32 + j])), w4[c * 32 + j], out);
  }
  return out;
}

__device__ __forceinline__ float run_net(Group& G, uint32_t w1, uint32_t w2, uint32_t w3, const float* f) {
  layer_mma(G, G.X, w1, kMlpIn);
  hidden_epilogue(G, f);
  layer_mma(G, G.H, w2, kMlpWidth);
  hidden_epilogue(G, f + kMlpWidth);
  layer_mma(G, G.H, w3, kMlpWidth);
  return output_epilogue(G, f);
}

__device__ __forceinline__ void write_x(Group& G, const float (&f)[kMlpIn]) {
  f16 x[kMlpIn];
  split_features(f, x);
  __align__(16) __half2 h[kMlpIn / 2];
#pragma unroll
  for (int i = 0; i < kMlpIn / 2; i++) {
    h[i].x = x[2 * i];
    h[i].y = x[2 * i + 1];
  }
  uint8_t* X = G.base + G.X;
  *reinterpret_cast<uint4*>(X + tc::tile_offset(G.lt, 0, kMlpIn)) = *reinterpret_cast<uint4*>(h);
  *reinterpret_cast<uint4*>(X + tc::tile_offset(G.lt, 8, kMlpIn)) = *reinterpret_cast<uint4*>(h + 4);
}

// inputs and outputs of one sampler launch: the array API (E, T per row,
// Philox uniforms keyed by the row, POD fallback outside the box) or the
// thermal-scatter queue (E, T and the particle's own two uniforms per row;
// rows are inside the box by construction, outputs in FP32)
struct SampleIO {
  const DevTSL* tsl;
  const double* E;
  const double* T;
  unsigned long long n;
  unsigned long long key;
  double* beta_out;
  double* alpha_out;
  unsigned long long* failures;
  const float4* qin;                 // queue form
  const unsigned long long* qcount;
  unsigned long long qcap;
  float2* qout;
};

template <bool QUEUE>
__global__ void __launch_bounds__(128 * kGroups, 1) k_mlp_sample(NetView nb, NetView na, MlpBox box, SampleIO io,
                                                                  int* err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  float* fb = reinterpret_cast<float*>(smem + kOffF);
  float* fa = fb + 4 * kMlpWidth + 4;
  uint32_t* misc = reinterpret_cast<uint32_t*>(smem + kOffMisc);  // [0..3] two mbarriers, [4] tensor memory
  const int tid = threadIdx.x, warp = tid >> 5;
  const unsigned long long n = QUEUE ? (*io.qcount < io.qcap ? *io.qcount : io.qcap) : io.n;
  if (n == 0) return;  // uniform across the grid: nothing allocated yet
  // weights into shared memory
  load_tile(smem + kOffB1, nb.W1, kMlpIn);
  load_tile(smem + kOffB2, nb.W2, kMlpWidth);
  load_tile(smem + kOffB3, nb.W3, kMlpWidth);
  load_tile(smem + kOffA1, na.W1, kMlpIn);
  load_tile(smem + kOffA2, na.W2, kMlpWidth);
  load_tile(smem + kOffA3, na.W3, kMlpWidth);
  for (int i = tid; i < kMlpWidth; i += blockDim.x) {  // hidden biases halved for the SiLU epilogues
    fb[i] = 0.5f * nb.p[kMlpB1 + i];
    fb[kMlpWidth + i] = 0.5f * nb.p[kMlpB2 + i];
    fb[2 * kMlpWidth + i] = 0.5f * nb.p[kMlpB3 + i];
    fb[3 * kMlpWidth + i] = nb.p[kMlpW4 + i];
    fa[i] = 0.5f * na.p[kMlpB1 + i];
    fa[kMlpWidth + i] = 0.5f * na.p[kMlpB2 + i];
    fa[2 * kMlpWidth + i] = 0.5f * na.p[kMlpB3 + i];
    fa[3 * kMlpWidth + i] = na.p[kMlpW4 + i];
  }
  if (tid == 0) {
    fb[4 * kMlpWidth] = nb.p[kMlpB4];
    fa[4 * kMlpWidth] = na.p[kMlpB4];
    for (int g = 0; g < kGroups; g++) tc::mbar_init(tc::smem_addr(misc + 2 * g), 1);
  }
  if (warp == 0) tc::tmem_alloc(tc::smem_addr(misc + 4), 128 * kGroups);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  Group G;
  G.base = smem;
  G.g = tid >> 7;
  G.lt = tid & 127;
  G.X = kOffG + G.g * kGroupBytes;
  G.H = G.X + kTileW1;
  G.tmem = misc[4] + 128 * G.g;
  G.mbar = tc::smem_addr(misc + 2 * G.g);
  G.phase = 0;
  G.ok = true;
  const double Emin = exp(box.logE0), Emax = exp(box.logE1);
  const BoxF bf = box_f(box);
  const float Eminf = static_cast<float>(Emin), T0f = static_cast<float>(box.T0);
  unsigned long long my_fail = 0;
  const unsigned long long tiles = (n + 127) / 128;
  const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * kGroups;
  for (unsigned long long tile = static_cast<unsigned long long>(blockIdx.x) * kGroups + G.g; tile < tiles && G.ok;
       tile += stride) {
    const unsigned long long i = tile * 128 + G.lt;
    const bool valid = i < n;
    float e, t, u1, u2;
    bool in_box = true;
    PhiloxRng rng;
    if constexpr (QUEUE) {
      const float4 q = valid ? io.qin[i] : make_float4(Eminf, T0f, 0.5f, 0.5f);
      e = q.x;
      t = q.y;
      u1 = q.z;
      u2 = q.w;
    }
    else {
      const double ed = valid ? io.E[i] : Emin;
      const double td = valid ? io.T[i] : box.T0;
      in_box = ed >= Emin && ed <= Emax && td >= box.T0 && td <= box.T1;
      // rows outside the box keep the tile's arithmetic finite and are resampled below
      e = in_box ? static_cast<float>(ed) : Eminf;
      t = in_box ? static_cast<float>(td) : T0f;
      rng.init(io.key, i, 3);
      u1 = rng.u01f();
      u2 = rng.u01f();
    }
    float x[kMlpIn];
    beta_features(bf, e, t, u1, x);
    write_x(G, x);
    const float qb = run_net(G, kOffB1, kOffB2, kOffB3, fb);
    const float bmin = beta_min_of(bf, e, t);
    const float b = fmaf(fminf(1.0f, fmaxf(0.0f, qb)), bf.beta_cutoff - bmin, bmin);
    alpha_features(bf, e, t, b, u2, x);
    write_x(G, x);
    const float qa = run_net(G, kOffA1, kOffA2, kOffA3, fa);
    float lo, hi;
    alpha_range(bf, e, t, b, lo, hi);
    const float a = fmaf(fminf(1.0f, fmaxf(0.0f, qa)), hi - lo, lo);
    if constexpr (QUEUE) {
      if (valid) io.qout[i] = make_float2(b, a);
    }
    else {
      double bo = b, ao = a;
      if (valid && !in_box) {
        // outside the trained box: the POD sampler (FP32 form when the ranks fit)
        const double eo = io.E[i], to = io.T[i];
        const DevTSL* tsl = io.tsl;
        bool ok = tsl->fast_ok ? tsl_sample_beta<true>(*tsl, rng, eo, to, bo)
                               : tsl_sample_beta<false>(*tsl, rng, eo, to, bo);
        if (ok) ok = tsl->fast_ok ? tsl_sample_alpha<true>(*tsl, rng, bo, eo, to, ao)
                                  : tsl_sample_alpha<false>(*tsl, rng, bo, eo, to, ao);
        if (!ok) {
          bo = ao = CUDART_NAN;
          my_fail++;
        }
      }
      if (valid) {
        io.beta_out[i] = bo;
        io.alpha_out[i] = ao;
      }
    }
  }
  if (!G.ok && G.lt == 0) atomicExch(err, 1);
  if constexpr (!QUEUE) {
    if (my_fail) atomicAdd(io.failures, my_fail);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(misc[4], 128 * kGroups);
  }
}

template <bool QUEUE>
cudaError_t sample_attr() {
  static bool attr = false;
  if (!attr) {
    const cudaError_t e =
        cudaFuncSetAttribute(k_mlp_sample<QUEUE>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSampleSmem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  return cudaSuccess;
}

}  // namespace

cudaError_t launch_sample_tsl_mlp(const DevTSL* tsl, const MlpNet& beta_net, const MlpNet& alpha_net,
                                  const MlpBox& box, const double* E, const double* T, unsigned long long n,
                                  unsigned long long key, double* beta, double* alpha, unsigned long long* failures,
                                  int num_sms, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  cudaError_t e = sample_attr<false>();
  if (e != cudaSuccess) return e;
  const unsigned long long tiles = (n + 127) / 128;
  const unsigned long long want = (tiles + kGroups - 1) / kGroups;
  const unsigned grid = static_cast<unsigned>(want < static_cast<unsigned long long>(num_sms) ? want : num_sms);
  NetView nb{beta_net.p, beta_net.W1, beta_net.W2, beta_net.W3};
  NetView na{alpha_net.p, alpha_net.W1, alpha_net.W2, alpha_net.W3};
  SampleIO io{};
  io.tsl = tsl;
  io.E = E;
  io.T = T;
  io.n = n;
  io.key = key;
  io.beta_out = beta;
  io.alpha_out = alpha;
  io.failures = failures;
  k_mlp_sample<false><<<grid, 128 * kGroups, kSampleSmem, s>>>(nb, na, box, io, mlp_err_ptr());
  return cudaGetLastError();
}

cudaError_t launch_sample_tsl_mlp_queue(const MlpNet& beta_net, const MlpNet& alpha_net, const MlpBox& box,
                                        const float4* qin, const unsigned long long* count, unsigned long long cap,
                                        float2* qout, int num_sms, cudaStream_t s) {
  if (cap == 0) return cudaSuccess;
  cudaError_t e = sample_attr<true>();
  if (e != cudaSuccess) return e;
  NetView nb{beta_net.p, beta_net.W1, beta_net.W2, beta_net.W3};
  NetView na{alpha_net.p, alpha_net.W1, alpha_net.W2, alpha_net.W3};
  SampleIO io{};
  io.qin = qin;
  io.qcount = count;
  io.qcap = cap;
  io.qout = qout;
  // the row count is known on the device only: one persistent CTA per SM
  k_mlp_sample<true><<<num_sms, 128 * kGroups, kSampleSmem, s>>>(nb, na, box, io, mlp_err_ptr());
  return cudaGetLastError();
}

int* mlp_error_flag() { return mlp_err_ptr(); }

// ---------------------------------------------------------------------------
// Learned brackets for SampleAlpha's CDF search (the guided sampler).
//
// ThermalScattering::SampleAlpha spends most of its time in find_cdf: a
// bisection over the CDF grid whose every probe is a rank-r POD
// reconstruction (src/ThermalScattering.cpp:395-421), twice per sample.  The
// guide network predicts where that search ends -- the grid position of the
// kinematic bound a, given |beta_s| and T -- and the search starts there:
// two reconstructions confirm a right guess, a wrong one is walked out with
// doubling steps and bisected (cdf_upper_guided).  Everything else is the
// POD sampler itself, so for the same random numbers the guided sampler
// returns exactly the POD sampler's (beta, alpha); only the work differs.

namespace {

// guide features of a bound a at |beta_s| and T (FP32, as in training):
// ln a, ln(1 + |beta|), T, the log ratio of a to |beta|, and the free-gas
// scaling variable (a - |beta|) / (2 sqrt a) -- for a free gas alpha given
// beta is close to normal in it -- plain and squashed
__device__ __forceinline__ void guide_features(const BoxF& b, float a, float abs_bs, float T, float (&f)[kMlpIn]) {
#pragma unroll
  for (int i = 0; i < kMlpIn; i++) f[i] = 0.0f;
  const float aa = fmaxf(a, 1e-12f);
  const float la = logf(aa);
  f[0] = fmaf(la, 0.1f, 1.0f);
  f[1] = fmaf(log1pf(abs_bs) * b.inv_beta_scale, 2.0f, -1.0f);
  f[2] = fmaf(T, b.t_scale, b.t_shift);
  f[3] = fminf(4.0f, fmaxf(-4.0f, (la - logf(abs_bs + 1e-3f)) * 0.125f));
  f[4] = aa / (aa + abs_bs + 1.0f);
  const float z = (aa - abs_bs) / (2.0f * sqrtf(aa));
  f[5] = fminf(4.0f, fmaxf(-4.0f, 0.25f * z));
  f[6] = tanhf(0.5f * z);
}

// training rows: per sample, (E, T) drawn in the box, beta from the POD
// sampler, the beta grid point SampleAlpha picks, and for each of the two
// bounds the features and the position where find_cdf's bisection ends
__global__ void k_guide_data(const DevTSL* tsl, MlpBox box, unsigned long long key, unsigned long long n, f16* X,
                             float* y, unsigned long long* failures) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const BoxF bf = box_f(box);
  const DevTSL& t = *tsl;
  PhiloxRng rng;
  rng.init(key, i, 6);
  const double E = exp(box.logE0 + rng.u01() * (box.logE1 - box.logE0));
  const double T = box.T0 + rng.u01() * (box.T1 - box.T0);
  double b = 0;
  AlphaCtx<true> x;
  const bool ok = tsl_sample_beta<true>(t, rng, E, T, b) && alpha_begin<true>(t, rng, b, E, T, x);
  float f[kMlpIn];
#pragma unroll 1
  for (int k = 0; k < 2; k++) {
    float target = 0.5f, a = 1.0f, bs = 1.0f;
    if (ok) {
      const double av = k == 0 ? x.b_s_a_min : x.b_s_a_max;
      target = cdf_position<true>(t, x, av, cdf_upper_bisect<true>(x, av));
      a = static_cast<float>(av);
      bs = fabsf(static_cast<float>(x.b_s));
    }
    guide_features(bf, a, bs, static_cast<float>(T), f);
    store_features(f, X + (2 * i + k) * kMlpIn);
    y[2 * i + k] = target;
  }
  if (!ok) atomicAdd(failures, 1ull);
}

constexpr int kGuideGroups = 4;  // warpgroups per CTA, each with its own tiles and accumulator
constexpr uint32_t kGOffW1 = 0;
constexpr uint32_t kGOffW2 = kGOffW1 + kTileW1;
constexpr uint32_t kGOffW3 = kGOffW2 + kTileW;
constexpr uint32_t kGOffG = kGOffW3 + kTileW;
constexpr uint32_t kGOffF = kGOffG + kGuideGroups * kGroupBytes;
constexpr uint32_t kGOffMisc = kGOffF + (4 * kMlpWidth + 4) * 4;
constexpr uint32_t kGuideSmem = kGOffMisc + 64;
static_assert(kGuideSmem <= 227 * 1024, "shared memory");

struct GuideIO {
  const DevTSL* tsl;
  // array form: (E, T) per row, Philox streams keyed by the row
  const double* E;
  const double* T;
  unsigned long long n;
  unsigned long long key;
  double* beta_out;
  double* alpha_out;
  unsigned long long* failures;
  // queue form: parked particles with their own streams
  const GuideRow* rows;
  const unsigned long long* qcount;
  unsigned long long qcap;
  unsigned long long run_key;
  GuideOut* qout;
};

// One thread per sample, 128-sample tiles per warpgroup: the POD SampleBeta
// and the beta grid choice on the CUDA cores, the guide network for both
// bounds on the tensor cores (one tcgen05 product per layer), then the
// guided searches and SampleAlpha's resampling loop.
template <bool QUEUE, bool FAST>
__global__ void __launch_bounds__(128 * kGuideGroups, 1) k_guided_sample(NetView nv, MlpBox box, GuideIO io, int* err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  float* fw = reinterpret_cast<float*>(smem + kGOffF);
  uint32_t* misc = reinterpret_cast<uint32_t*>(smem + kGOffMisc);  // [0, 2G) mbarriers, [2G] tensor memory
  const int tid = threadIdx.x, warp = tid >> 5;
  const unsigned long long n = QUEUE ? (*io.qcount < io.qcap ? *io.qcount : io.qcap) : io.n;
  if (n == 0) return;  // uniform across the grid: nothing allocated yet
  load_tile(smem + kGOffW1, nv.W1, kMlpIn);
  load_tile(smem + kGOffW2, nv.W2, kMlpWidth);
  load_tile(smem + kGOffW3, nv.W3, kMlpWidth);
  for (int i = tid; i < kMlpWidth; i += blockDim.x) {  // hidden biases halved for the SiLU epilogues
    fw[i] = 0.5f * nv.p[kMlpB1 + i];
    fw[kMlpWidth + i] = 0.5f * nv.p[kMlpB2 + i];
    fw[2 * kMlpWidth + i] = 0.5f * nv.p[kMlpB3 + i];
    fw[3 * kMlpWidth + i] = nv.p[kMlpW4 + i];
  }
  if (tid == 0) {
    fw[4 * kMlpWidth] = nv.p[kMlpB4];
    for (int g = 0; g < kGuideGroups; g++) tc::mbar_init(tc::smem_addr(misc + 2 * g), 1);
  }
  if (warp == 0) tc::tmem_alloc(tc::smem_addr(misc + 2 * kGuideGroups), 128 * kGuideGroups);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  Group G;
  G.base = smem;
  G.g = tid >> 7;
  G.lt = tid & 127;
  G.X = kGOffG + G.g * kGroupBytes;
  G.H = G.X + kTileW1;
  G.tmem = misc[2 * kGuideGroups] + 128 * G.g;
  G.mbar = tc::smem_addr(misc + 2 * G.g);
  G.phase = 0;
  G.ok = true;
  const BoxF bf = box_f(box);
  const DevTSL& t = *io.tsl;
  unsigned long long my_fail = 0;
  const unsigned long long tiles = (n + 127) / 128;
  const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * kGuideGroups;
  for (unsigned long long tile = static_cast<unsigned long long>(blockIdx.x) * kGuideGroups + G.g;
       tile < tiles && G.ok; tile += stride) {
    const unsigned long long i = tile * 128 + G.lt;
    const bool valid = i < n;
    PhiloxRng rng;
    double E = 1e-7, T = 300.0;
    if constexpr (QUEUE) {
      if (valid) {
        const GuideRow R = io.rows[i];
        E = R.E;
        T = R.T;
        rng.restore(io.run_key, R.rng_id, R.rng_tag, R.rng_pos);
      }
    }
    else {
      if (valid) {
        E = io.E[i];
        T = io.T[i];
      }
      rng.init(io.key, i, 2);
    }
    double b = 0, a_min = 1.0, a_max = 1.0;
    float abs_bs = 1.0f;
    int b_s_i = -1;
    bool ok = valid && tsl_sample_beta<FAST>(t, rng, E, T, b);
    if (ok) {
      AlphaCtx<FAST> x;
      ok = alpha_begin<FAST>(t, rng, b, E, T, x);
      if (ok) {
        b_s_i = x.b_s_i;
        a_min = x.b_s_a_min;
        a_max = x.b_s_a_max;
        abs_bs = fabsf(static_cast<float>(x.b_s));
      }
    }
    // the guide network on both bounds (every row of the tile takes part)
    float f[kMlpIn];
    guide_features(bf, static_cast<float>(a_min), abs_bs, static_cast<float>(T), f);
    write_x(G, f);
    const float q0 = run_net(G, kGOffW1, kGOffW2, kGOffW3, fw);
    guide_features(bf, static_cast<float>(a_max), abs_bs, static_cast<float>(T), f);
    write_x(G, f);
    const float q1 = run_net(G, kGOffW1, kGOffW2, kGOffW3, fw);
    double alpha = 0;
    if (ok) {
      AlphaCtx<FAST> x;
      alpha_setup<FAST>(t, b, E, T, b_s_i, x);  // the same context, rebuilt after the network
      const float m = static_cast<float>(x.nF + 1);
      const int g0 = static_cast<int>(floorf(fminf(1.0f, fmaxf(0.0f, q0)) * m));
      const int g1 = static_cast<int>(floorf(fminf(1.0f, fmaxf(0.0f, q1)) * m));
      // grid points whose reconstruction is not safely monotone, and
      // temperatures outside the tabulated range (where Evaluate
      // extrapolates), keep the bisection, so the answer is always the POD
      // sampler's
      const bool mono = (__ldg(t.alpha.mono + b_s_i) & (FAST ? 1 : 2)) != 0 && x.ev.c.Tl < x.ev.c.Th &&
                        x.ev.c.Tl <= T && T <= x.ev.c.Th;
      Probes p0, p1;  // each guided search's last reconstructions, reused by cdf_at
      const int i_min =
          mono ? cdf_upper_guided_kept<FAST>(x, x.b_s_a_min, g0, p0) : cdf_upper_bisect<FAST>(x, x.b_s_a_min);
      const int i_max =
          mono ? cdf_upper_guided_kept<FAST>(x, x.b_s_a_max, g1, p1) : cdf_upper_bisect<FAST>(x, x.b_s_a_max);
      const double F_min = cdf_at_kept<FAST>(t, x, x.b_s_a_min, i_min, p0);
      const double F_max = cdf_at_kept<FAST>(t, x, x.b_s_a_max, i_max, p1);
      ok = alpha_end<FAST>(t, rng, x, F_min, F_max, alpha);
    }
    if (valid) {
      if constexpr (QUEUE) {
        GuideOut o;
        o.beta = ok ? b : CUDART_NAN;
        o.alpha = ok ? alpha : CUDART_NAN;
        o.rng_pos = rng.save();
        o.ok = ok ? 1 : 0;
        io.qout[i] = o;
      }
      else {
        io.beta_out[i] = ok ? b : CUDART_NAN;
        io.alpha_out[i] = ok ? alpha : CUDART_NAN;
        if (!ok) my_fail++;
      }
    }
  }
  if (!G.ok && G.lt == 0) atomicExch(err, 1);
  if constexpr (!QUEUE) {
    if (my_fail) atomicAdd(io.failures, my_fail);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(misc[2 * kGuideGroups], 128 * kGuideGroups);
  }
}

// the POD sampler on the same queue, without the network (the ablation of
// the guided form: same batching, find_cdf by plain bisection)
template <bool FAST>
__global__ void __launch_bounds__(256) k_pod_queue(const DevTSL* tsl, const GuideRow* rows,
                                                   const unsigned long long* qcount, unsigned long long qcap,
                                                   unsigned long long run_key, GuideOut* qout) {
  const unsigned long long n = *qcount < qcap ? *qcount : qcap;
  for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    const GuideRow R = rows[i];
    PhiloxRng rng;
    rng.restore(run_key, R.rng_id, R.rng_tag, R.rng_pos);
    double b = 0, a = 0;
    const bool ok =
        tsl_sample_beta<FAST>(*tsl, rng, R.E, R.T, b) && tsl_sample_alpha<FAST>(*tsl, rng, b, R.E, R.T, a);
    GuideOut o;
    o.beta = ok ? b : CUDART_NAN;
    o.alpha = ok ? a : CUDART_NAN;
    o.rng_pos = rng.save();
    o.ok = ok ? 1 : 0;
    qout[i] = o;
  }
}

template <bool QUEUE, bool FAST>
cudaError_t guided_attr() {
  static bool attr = false;
  if (!attr) {
    const cudaError_t e =
        cudaFuncSetAttribute(k_guided_sample<QUEUE, FAST>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGuideSmem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  return cudaSuccess;
}

}  // namespace

cudaError_t launch_guide_data(const DevTSL* tsl, const MlpBox& box, unsigned long long key, unsigned long long n,
                              __half* X, float* y, unsigned long long* failures, cudaStream_t s) {
  k_guide_data<<<blocks256(n), 256, 0, s>>>(tsl, box, key, n, X, y, failures);
  return cudaGetLastError();
}

cudaError_t launch_sample_tsl_guided(const DevTSL* tsl, const MlpNet& guide, const MlpBox& box, bool fast,
                                     const double* E, const double* T, unsigned long long n, unsigned long long key,
                                     double* beta, double* alpha, unsigned long long* failures, int num_sms,
                                     cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  cudaError_t e = fast ? guided_attr<false, true>() : guided_attr<false, false>();
  if (e != cudaSuccess) return e;
  const unsigned long long tiles = (n + 127) / 128;
  const unsigned long long want = (tiles + kGuideGroups - 1) / kGuideGroups;
  const unsigned grid = static_cast<unsigned>(want < static_cast<unsigned long long>(num_sms) ? want : num_sms);
  NetView nv{guide.p, guide.W1, guide.W2, guide.W3};
  GuideIO io{};
  io.tsl = tsl;
  io.E = E;
  io.T = T;
  io.n = n;
  io.key = key;
  io.beta_out = beta;
  io.alpha_out = alpha;
  io.failures = failures;
  if (fast) k_guided_sample<false, true><<<grid, 128 * kGuideGroups, kGuideSmem, s>>>(nv, box, io, mlp_err_ptr());
  else k_guided_sample<false, false><<<grid, 128 * kGuideGroups, kGuideSmem, s>>>(nv, box, io, mlp_err_ptr());
  return cudaGetLastError();
}

cudaError_t launch_sample_tsl_guided_queue(const DevTSL* tsl, const MlpNet& guide, const MlpBox& box, bool fast,
                                           const GuideRow* rows, const unsigned long long* count,
                                           unsigned long long cap, unsigned long long run_key, GuideOut* out,
                                           int num_sms, cudaStream_t s) {
  if (cap == 0) return cudaSuccess;
  cudaError_t e = fast ? guided_attr<true, true>() : guided_attr<true, false>();
  if (e != cudaSuccess) return e;
  NetView nv{guide.p, guide.W1, guide.W2, guide.W3};
  GuideIO io{};
  io.tsl = tsl;
  io.rows = rows;
  io.qcount = count;
  io.qcap = cap;
  io.run_key = run_key;
  io.qout = out;
  // the row count is known on the device only: one persistent CTA per SM
  if (fast) k_guided_sample<true, true><<<num_sms, 128 * kGuideGroups, kGuideSmem, s>>>(nv, box, io, mlp_err_ptr());
  else k_guided_sample<true, false><<<num_sms, 128 * kGuideGroups, kGuideSmem, s>>>(nv, box, io, mlp_err_ptr());
  return cudaGetLastError();
}

cudaError_t launch_sample_tsl_pod_queue(const DevTSL* tsl, bool fast, const GuideRow* rows,
                                        const unsigned long long* count, unsigned long long cap,
                                        unsigned long long run_key, GuideOut* out, int num_sms, cudaStream_t s) {
  if (cap == 0) return cudaSuccess;
  if (fast) k_pod_queue<true><<<num_sms * 8, 256, 0, s>>>(tsl, rows, count, cap, run_key, out);
  else k_pod_queue<false><<<num_sms * 8, 256, 0, s>>>(tsl, rows, count, cap, run_key, out);
  return cudaGetLastError();
}

}  // namespace mcd

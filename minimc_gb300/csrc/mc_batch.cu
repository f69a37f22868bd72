// Batched multigroup k-eigenvalue problems: per-cycle bookkeeping kernels.
//
// All problems' histories are concatenated (problem p owns histories
// off[p] .. off[p+1]), so the fission-bank prefix sum and compaction run
// once over all of them and problem p's bank is the contiguous range its
// histories produced, in history order.  Keys, bank sizes, k and the
// resampling index are computed on the device from a device-resident cycle
// counter, so one cycle's launches form a static CUDA graph.  Per problem
// the keys and draws are those of a single-problem run
// (mc_keig_cycle): a problem gives the same k per cycle batched or alone.
#include "mc_kernels.cuh"

namespace mcd {

namespace {

__device__ __forceinline__ unsigned long long dev_run_key(unsigned long long seed, unsigned long long cycle,
                                                          unsigned long long salt) {
  return splitmix64(seed * 0x9E3779B97F4A7C15ull + cycle * 0xD1B54A32D192ED03ull + salt);
}

__global__ void k_batch_begin(const BatchCycle b, const Site* src) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= b.P) return;
  const unsigned long long c = *b.cycle;
  RunParams& rp = b.rps[p];
  rp.cycle = static_cast<uint32_t>(c);
  rp.run_key = dev_run_key(b.seeds[p], c, 0x4b454947ull);
  rp.minstd_base = b.seeds[p] + c * rp.n;
  rp.from_bank = c > 0 ? 1 : 0;
  rp.src = src + b.off[p];
  b.ctr[p] = DevCounters{};
}

__global__ void k_batch_tally(const BatchCycle b, const unsigned long long* offsets, const unsigned long long* total) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= b.P) return;
  const unsigned long long s = offsets[b.off[p]];
  const unsigned long long e = p + 1 < b.P ? offsets[b.off[p + 1]] : *total;
  const unsigned long long m = e - s;
  const unsigned c = *b.cycle;
  b.start[p] = s;
  b.M[p] = m;
  if (c < static_cast<unsigned>(b.max_cycles))
    b.k[static_cast<size_t>(p) * b.max_cycles + c] = static_cast<double>(m) / static_cast<double>(b.off[p + 1] - b.off[p]);
  if (m == 0) *b.died = 1;
  unsigned long long* st = b.stats + 4 * p;
  st[0] += b.ctr[p].events;
  st[1] += b.ctr[p].lost;
  st[2] += b.ctr[p].capped;
  st[3] += b.ctr[p].overflow;
}

// next source j of problem p = bank[start_p + floor(U_j * M_p)], U_j from
// Philox(run key of (seed_p, cycle), counter j) as the single-problem
// resampler draws it
__global__ void k_batch_resample(const BatchCycle b, const Site* bank, Site* next) {
  const unsigned long long j = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= b.N) return;
  int lo = 0, hi = b.P;  // last p with off[p] <= j
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (b.off[mid] <= j) lo = mid;
    else hi = mid;
  }
  const int p = lo;
  const unsigned long long jj = j - b.off[p];
  const unsigned long long m = b.M[p];
  if (m == 0) return;
  const unsigned long long key = dev_run_key(b.seeds[p], *b.cycle, 0x52455341ull);
  next[j] = bank[b.start[p] + resample_index(key, jj, m)];
}

__global__ void k_batch_next_cycle(const BatchCycle b) { *b.cycle += 1; }

__global__ void k_keig_record(const DevCounters* ctr, unsigned long long* total, unsigned long long n,
                              double* out, DevCounters* acc) {
  const DevCounters& c = *ctr;
  const unsigned long long m = *total;
  out[0] = static_cast<double>(m) / static_cast<double>(n);
  out[1] = static_cast<double>(m);
  out[2] = c.k_tracklength / static_cast<double>(n);
  if (c.lost && !acc->lost) {
    for (int i = 0; i < 3; i++) acc->lost_xyz[i] = c.lost_xyz[i];
    for (int i = 0; i < 4; i++) acc->pad[i] = c.pad[i];
  }
  acc->events += c.events;
  acc->secondaries += c.secondaries;
  acc->lost += c.lost;
  acc->capped += c.capped;
  acc->overflow += c.overflow;
  acc->resample += c.resample;
  acc->banked += c.banked;
  acc->k_tracklength += c.k_tracklength;
  if (m == 0) {  // a cycle's bank came out empty
    acc->next = 1;
    *total = 1;
  }
}

unsigned blocks_for(unsigned long long n) { return static_cast<unsigned>((n + 255) / 256); }

}  // namespace

cudaError_t launch_batch_begin(const BatchCycle& b, const Site* src, cudaStream_t s) {
  k_batch_begin<<<blocks_for(b.P), 256, 0, s>>>(b, src);
  return cudaGetLastError();
}

cudaError_t launch_batch_tally(const BatchCycle& b, const unsigned long long* offsets,
                               const unsigned long long* total, cudaStream_t s) {
  k_batch_tally<<<blocks_for(b.P), 256, 0, s>>>(b, offsets, total);
  return cudaGetLastError();
}

cudaError_t launch_keig_record(const DevCounters* ctr, unsigned long long* total, unsigned long long n,
                               double* out, DevCounters* acc, cudaStream_t stream) {
  k_keig_record<<<1, 1, 0, stream>>>(ctr, total, n, out, acc);
  return cudaGetLastError();
}

cudaError_t launch_batch_resample(const BatchCycle& b, const Site* bank, Site* next, cudaStream_t s) {
  k_batch_resample<<<blocks_for(b.N), 256, 0, s>>>(b, bank, next);
  k_batch_next_cycle<<<1, 1, 0, s>>>(b);
  return cudaGetLastError();
}

}  // namespace mcd

// FP32-table continuous-energy history kernels, occupancy variants MINB = 4,
// 5 and 6 (Philox streams in fast mode; see mc_history_ce.cuh).
#include "mc_history_ce.cuh"

namespace mcd {
namespace cevar {

namespace {
template <int MINB>
int occ(int block, bool keig) {
  return keig ? occupancy_of(k_history_ce<PhiloxRng, true, MINB, true>, block, kCeSmem)
              : occupancy_of(k_history_ce<PhiloxRng, false, MINB, true>, block, kCeSmem);
}
template <int MINB>
void run(const DevWorld& w, const RunParams& rp, int grid, int block, cudaStream_t stream) {
  if (rp.keig) k_history_ce<PhiloxRng, true, MINB, true><<<grid, block, kCeSmem, stream>>>(w, rp);
  else k_history_ce<PhiloxRng, false, MINB, true><<<grid, block, kCeSmem, stream>>>(w, rp);
}
}  // namespace

int occupancy_fx2(int minb, int block, bool keig) {
  return minb == 6 ? occ<6>(block, keig) : minb == 5 ? occ<5>(block, keig) : occ<4>(block, keig);
}

void launch_fx2(int minb, const DevWorld& w, const RunParams& rp, int grid, int block, cudaStream_t stream) {
  if (minb == 6) run<6>(w, rp, grid, block, stream);
  else if (minb == 5) run<5>(w, rp, grid, block, stream);
  else run<4>(w, rp, grid, block, stream);
}

}  // namespace cevar
}  // namespace mcd

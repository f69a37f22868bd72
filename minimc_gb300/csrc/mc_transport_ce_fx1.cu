// FP32-table continuous-energy history kernels, occupancy variants MINB = 1
// and 3 (Philox streams in fast mode; see mc_history_ce.cuh).
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

bool has_fx1(int minb) { return minb == 1 || minb == 3; }

int occupancy_fx1(int minb, int block, bool keig) { return minb == 3 ? occ<3>(block, keig) : occ<1>(block, keig); }

void launch_fx1(int minb, const DevWorld& w, const RunParams& rp, int grid, int block, cudaStream_t stream) {
  if (minb == 3) run<3>(w, rp, grid, block, stream);
  else run<1>(w, rp, grid, block, stream);
}

}  // namespace cevar
}  // namespace mcd

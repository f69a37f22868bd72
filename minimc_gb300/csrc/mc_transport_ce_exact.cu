// Exact-table continuous-energy history kernels (reference rounding), both
// stream families (see mc_history_ce.cuh).
#include "mc_history_ce.cuh"

namespace mcd {
namespace cevar {

int occupancy_exact(int rng_mode, int block, bool keig) {
  if (rng_mode == 1) return keig ? occupancy_of(k_history_ce<MinstdRng, true, 1, false>, block, kCeSmem)
                                 : occupancy_of(k_history_ce<MinstdRng, false, 1, false>, block, kCeSmem);
  return keig ? occupancy_of(k_history_ce<PhiloxRng, true, 1, false>, block, kCeSmem)
              : occupancy_of(k_history_ce<PhiloxRng, false, kExactFixedMinb, false>, block, kCeSmem);
}

void launch_exact(const DevWorld& w, const RunParams& rp, int rng_mode, int grid, int block, cudaStream_t stream) {
  if (rng_mode == 1) {
    if (rp.keig) k_history_ce<MinstdRng, true, 1, false><<<grid, block, kCeSmem, stream>>>(w, rp);
    else k_history_ce<MinstdRng, false, 1, false><<<grid, block, kCeSmem, stream>>>(w, rp);
  }
  else {
    if (rp.keig) k_history_ce<PhiloxRng, true, 1, false><<<grid, block, kCeSmem, stream>>>(w, rp);
    else k_history_ce<PhiloxRng, false, kExactFixedMinb, false><<<grid, block, kCeSmem, stream>>>(w, rp);
  }
}

}  // namespace cevar
}  // namespace mcd

// Continuous-energy history kernels with indirect effects of perturbations
// (fixed source, exact tables) and with the thermal-scatter queue (fixed
// source, Philox streams); see mc_history_ce.cuh.
#include "mc_history_ce.cuh"

namespace mcd {
namespace cevar {

void launch_pert(const DevWorld& w, const RunParams& rp, int rng_mode, int grid, int block, cudaStream_t stream) {
  if (rng_mode == 1) k_history_ce<MinstdRng, false, 1, false, true><<<grid, block, kCeSmem, stream>>>(w, rp);
  else k_history_ce<PhiloxRng, false, 1, false, true><<<grid, block, kCeSmem, stream>>>(w, rp);
}

void launch_tq(const DevWorld& w, const RunParams& rp, int grid, int block, cudaStream_t stream) {
  k_history_ce<PhiloxRng, false, kExactFixedMinb, false, false, true><<<grid, block, kCeSmem, stream>>>(w, rp);
}

}  // namespace cevar
}  // namespace mcd

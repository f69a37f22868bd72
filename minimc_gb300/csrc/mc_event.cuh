// Event-schedule data structures (mc_event.cu).
#pragma once

#include "mc_kernels.cuh"

namespace mcd {

// most bins an event-schedule run keeps per history (dense pending scores);
// problems with more bins use the history schedule
constexpr int kEvDenseBins = kDenseBins;

// structure-of-arrays particle store
struct EvState {
  double *x, *y, *z, *u, *v, *w;
  double* E;            // continuous energy (MeV)
  int32_t* g;           // multigroup group, 0-based
  int32_t* cell;
  int32_t* skip;        // robust crossing: surface just left
  uint32_t* nev;        // events of this particle
  uint32_t* hist;       // owning history
  unsigned long long* id;  // Philox particle id
  uint32_t* rng;        // saved stream position (PhiloxRng/MinstdRng::save)
  uint8_t* tag;         // bit 0: secondary, bit 1: photon
};

struct EvParams {
  RunParams rp;
  EvState st;
  unsigned capacity;  // particle slots
  int32_t* q_in;
  int32_t* q_out;
  int32_t* q_coll;
  unsigned* cnt;      // [0] in, [1] out, [2] collisions, [3] slots used,
                      // [4] 1 when this step's collision queue was sorted
  // Collision-queue ordering: when sort_keys > 0 and a step's collision
  // queue holds at least sort_min particles, it is counting-sorted by
  // (particle type, material, group) into q_sorted before the collide
  // kernel, so neighbouring lanes read the same cross-section rows.  Every
  // particle draws from its own stream, so the order changes no result.
  int32_t* q_sorted;
  unsigned* sort_hist;  // [2 * kEvSortKeys]: counts, then write positions
  unsigned sort_min;
  int32_t sort_keys;
};

constexpr int kEvSortKeys = 256;  // most (type, material, group) keys the sort handles

struct EvLaunch {
  int grid;
  unsigned max_iterations;
  unsigned check_every;  // iterations between host checks of the queue size
};

// callback after kernel launches (counts launches); may be null
typedef void (*EvStepHook)(void* ctx, int launches);

cudaError_t launch_event_mg(const DevWorld& w, const EvParams& ep, const EvLaunch& L, int rng_mode,
                            cudaStream_t stream, EvStepHook hook, void* hook_ctx);

}  // namespace mcd

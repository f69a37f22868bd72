// Deterministic geometry kernels exposed through the C ABI so that parity
// tests can compare them bit-for-bit with the CPU oracle:
// World::FindCellContaining, Cell::NearestSurface, CSGSurface::Distance and
// CSGSurface::Contains, one query per thread; and the continuous-energy
// material cross sections and energy-grid search.
#include "mc_ce.cuh"
#include "mc_kernels.cuh"

namespace mcd {

namespace {

__global__ void k_find_cell(const DevWorld w, const double* xyz, unsigned long long n, int32_t* cell) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  cell[i] = find_cell(w, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
}

__global__ void k_nearest_surface(const DevWorld w, const int32_t* cell, const double* xyz, const double* uvw,
                                  unsigned long long n, int32_t* surf, double* dist) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = cell[i];
  if (c < 0 || c >= w.n_cells) {
    surf[i] = -1;
    dist[i] = CUDART_INF;
    return;
  }
  double d;
  surf[i] = nearest_surface(w, c, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], uvw[3 * i], uvw[3 * i + 1],
                            uvw[3 * i + 2], d);
  dist[i] = d;
}

__global__ void k_surface_distance(const DevWorld w, int32_t s, const double* xyz, const double* uvw,
                                   unsigned long long n, double* dist) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dist[i] = surface_distance(w, s, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], uvw[3 * i], uvw[3 * i + 1],
                             uvw[3 * i + 2]);
}

__global__ void k_surface_contains(const DevWorld w, int32_t s, const double* xyz, unsigned long long n, int8_t* out) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = surface_contains(w, s, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]) ? 1 : 0;
}

// Material::GetMicroscopicTotal / GetMicroscopicMajorant for a neutron in
// `cell` (multigroup: energy holds the group number)
__global__ void k_material_xs_mg(const DevWorld w, int32_t cell, const double* energy, unsigned long long n,
                                 double* total, double* majorant) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int m = __ldg(w.cell_mat + cell);
  const int g = static_cast<int>(energy[i]) - 1;
  double t = 0;
  if (m >= 0 && g >= 0 && g < w.G) t = __ldg(w.mat_mg_total + static_cast<size_t>(m) * w.G + g);
  total[i] = t;
  majorant[i] = t;  // Multigroup::GetMajorant returns the total
}

// Material::GetMicroscopicTotal / GetMicroscopicMajorant of a
// continuous-energy neutron at a point of the cell (exact tables)
__global__ void k_material_xs_ce(const DevWorld w, int32_t cell, const double* energy, const double* xyz,
                                 unsigned long long n, double* total, double* majorant) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double E = energy[i];
  const int j = ce_search(w.ce, E);
  const int m = __ldg(w.cell_mat + cell);
  const double T = cell_temperature(w, cell, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
  total[i] = ce_material_micro(w, m, 0, j, E, T, T, false);
  majorant[i] = ce_material_micro(w, m, 0, j, E, cell_temperature_max(w, cell), T, true);
}

// std::map::upper_bound position of each energy in each table of a nuclide,
// found through the union grid: columns total, reactions in input order,
// nubar tables of the fission reactions, -1 past the last table
__global__ void k_energy_index(const DevWorld w, int32_t nuc, const double* energy, unsigned long long n,
                               long long* out) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const mc::CENuclideDesc& d = ce_desc(w, 0, nuc);
  const int j = ce_search(w.ce, energy[i]);
  long long* o = out + 6 * i;
  int col = 0;
  o[col++] = ce_table_index(w.ce, d.total, j);
  for (int k = 0; k < d.n_rx; k++) o[col++] = ce_table_index(w.ce, d.rx_table[k], j);
  for (int k = 0; k < d.n_rx && col < 6; k++)
    if (d.rx_nubar[k] >= 0) o[col++] = ce_table_index(w.ce, d.rx_nubar[k], j);
  while (col < 6) o[col++] = -1;
}

unsigned blocks_for(unsigned long long n) { return static_cast<unsigned>((n + 255) / 256); }

}  // namespace

cudaError_t launch_find_cell(const DevWorld& w, const double* xyz, unsigned long long n, int32_t* cell,
                             cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  k_find_cell<<<blocks_for(n), 256, 0, stream>>>(w, xyz, n, cell);
  return cudaGetLastError();
}

cudaError_t launch_nearest_surface(const DevWorld& w, const int32_t* cell, const double* xyz, const double* uvw,
                                   unsigned long long n, int32_t* surf, double* dist, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  k_nearest_surface<<<blocks_for(n), 256, 0, stream>>>(w, cell, xyz, uvw, n, surf, dist);
  return cudaGetLastError();
}

cudaError_t launch_surface_distance(const DevWorld& w, int32_t s, const double* xyz, const double* uvw,
                                    unsigned long long n, double* dist, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  k_surface_distance<<<blocks_for(n), 256, 0, stream>>>(w, s, xyz, uvw, n, dist);
  return cudaGetLastError();
}

cudaError_t launch_surface_contains(const DevWorld& w, int32_t s, const double* xyz, unsigned long long n,
                                    int8_t* out, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  k_surface_contains<<<blocks_for(n), 256, 0, stream>>>(w, s, xyz, n, out);
  return cudaGetLastError();
}

cudaError_t launch_material_xs_mg(const DevWorld& w, int32_t cell, const double* energy, unsigned long long n,
                                  double* total, double* majorant, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  k_material_xs_mg<<<blocks_for(n), 256, 0, stream>>>(w, cell, energy, n, total, majorant);
  return cudaGetLastError();
}

cudaError_t launch_material_xs_ce(const DevWorld& w, int32_t cell, const double* energy, const double* xyz,
                                  unsigned long long n, double* total, double* majorant, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  k_material_xs_ce<<<blocks_for(n), 256, 0, stream>>>(w, cell, energy, xyz, n, total, majorant);
  return cudaGetLastError();
}

cudaError_t launch_energy_index(const DevWorld& w, int32_t nuclide, const double* energy, unsigned long long n,
                                long long* out, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  k_energy_index<<<blocks_for(n), 256, 0, stream>>>(w, nuclide, energy, n, out);
  return cudaGetLastError();
}

}  // namespace mcd

// Host-side problem model: the minimc XML input turned into flat tables.
//
// This plays the role of minimc's World (reference src/World.cpp:20-24), its
// CSGSurface/Cell/Material/Nuclide/ScalarField objects, the Source
// (src/Source.cpp:143-154), the Driver settings (src/Driver.cpp:37-52) and the
// EstimatorSet (src/Estimator.cpp:185-205).  Everything is stored as indices
// and contiguous arrays so that it can be uploaded to the device unchanged.
//
// Object order follows the reference's construction order:
//   * surfaces, materials and nuclides are numbered in order of first
//     appearance while walking <cells> (World::CreateCSGSurfaces,
//     CreateMaterials, CreateNuclides, src/World.cpp:98-170);
//   * a cell's surfaces and a material's nuclides are kept sorted by that
//     creation number.  The reference keys both in std::map by shared_ptr
//     address (src/Cell.hpp:30, src/Material.hpp:20), which is creation order
//     whenever the heap hands out ascending addresses.  The order matters for
//     tie-breaking in Cell::NearestSurface and for the nuclide CDF in
//     Particle::SampleNuclide.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace mc {

// Kinds of CSG surface.  sphere/planex/cylinderx are the reference's own
// (src/CSGSurface.hpp:52-56); planey/planez/cylindery/cylinderz are
// extensions with the same conventions.
enum SurfaceKind : int32_t {
  kSphere = 0,
  kPlaneX = 1,
  kPlaneY = 2,
  kPlaneZ = 3,
  kCylinderX = 4,
  kCylinderY = 5,
  kCylinderZ = 6,
};

enum ParticleType : int32_t { kNeutron = 0, kPhoton = 1 };
enum Tracking : int32_t { kSurfaceTracking = 0, kCellDeltaTracking = 1 };
enum ProblemType : int32_t { kFixedSource = 0, kKEigenvalue = 1 };
enum EnergyMode : int32_t { kMultigroup = 0, kContinuous = 1 };
enum ReactionKind : int32_t { kCapture = 0, kScatter = 1, kFission = 2 };
enum EstimatorKind : int32_t { kCurrent = 0, kTrackLength = 1 };
enum BinKind : int32_t { kNoBins = 0, kLinspace = 1, kLogspace = 2, kBoundaries = 3 };
enum DirectionDist : int32_t { kDirConstant = 0, kDirIsotropic = 1, kDirIsotropicFlux = 2 };

struct Surface {
  std::string name;
  int32_t kind = kSphere;
  int32_t reflective = 0;  // extension: 1 = specular reflection boundary
  // sphere: center (p[0..2]) and radius p[3]; plane: position p[0];
  // cylinder: radius p[0]
  double p[4] = {0, 0, 0, 0};
};

// ScalarField (src/ScalarField.hpp): constant c, or linear g.p + b with
// user-given bounds.
struct ScalarField {
  int32_t linear = 0;
  double c = 0;
  double g[3] = {0, 0, 0};
  double b = 0;
  double upper = 0, lower = 0;
  bool IsConstant() const { return !linear || (g[0] == 0 && g[1] == 0 && g[2] == 0); }
  double at(double x, double y, double z) const { return linear ? g[0] * x + g[1] * y + g[2] * z + b : c; }
};

struct Cell {
  std::string name;
  int32_t material = -1;  // -1: void (src/Cell.cpp:91-93)
  int32_t temperature = 0;  // index into Model::fields
  std::vector<int32_t> surfaces;  // sorted by surface creation number
  std::vector<uint8_t> within;    // 1: sense "-1" (cell on the negative side)
};

// Multigroup data for one (nuclide, particle type) (src/Multigroup.cpp).
// Matrices are stored by incoming group: m[(g_in-1)*G + (g_out-1)], columns
// normalized to unit sum as NormalizedTwoDimensional does (:168-186).
struct MGData {
  bool has_capture = false, has_scatter = false, has_fission = false;
  std::vector<double> capture, scatter, fission, total;  // [G]
  std::vector<double> scatter_prob;                       // [G*G]
  std::vector<double> nubar;                              // [G]
  std::vector<double> chi;                                // [G*G]
};

// One tabulated function of energy (ContinuousMap over an HDF5 axis).
struct Table1D {
  std::vector<double> x, y;
};

// ContinuousEvaluation (src/ContinuousEvaluation.hpp).
struct CEEval {
  Table1D xs;
  double temperature = 0;
  bool IsValid(double requested) const;
};

// Proper-orthogonal-decomposition thermal scattering tables
// (src/ThermalScattering.hpp:58-127), partitions concatenated.
struct PODPartitionSet {
  // per partition
  std::vector<std::vector<double>> F;       // CDF axis (level 0 of CDF_modes)
  std::vector<std::vector<double>> cdf_modes;  // [nF][rank]
  std::vector<std::vector<double>> S;       // [rank]
  std::vector<std::vector<double>> grid;    // E (beta partitions) or beta (alpha partitions)
  std::vector<std::vector<double>> T;       // temperature axis (level 1)
  std::vector<std::vector<double>> g_t_modes;  // [n_grid][nT][rank]
  std::vector<double> concat;               // Es or betas, concatenated
  std::vector<size_t> ends;                 // one-past-the-last index per partition
};

struct TSLData {
  Table1D majorant;
  std::vector<double> xs_T;      // T axis of total_T
  std::vector<double> xs_T_modes;  // [nT][rank]
  std::vector<double> xs_S;      // [rank]
  std::vector<double> xs_E;      // E axis of total_E
  std::vector<double> xs_E_modes;  // [nE][rank]
  size_t xs_rank = 0;
  PODPartitionSet beta, alpha;
  double beta_cutoff = 0, alpha_cutoff = 0, awr = 0;
  double cutoff_energy() const { return xs_E.empty() ? 0 : xs_E.back(); }
};

struct CEReaction {
  int32_t kind = kCapture;
  CEEval eval;
  int32_t tsl = -1;  // index into Model::tsl (scatter only)
  bool has_nubar = false;
  Table1D nubar;     // fission only
};

struct CEData {
  double awr = 0;
  CEEval total;
  std::vector<CEReaction> reactions;  // XML order, "total" excluded
};

struct Nuclide {
  std::string name;
  // indexed by particle type (kNeutron, kPhoton); present[t] tells whether
  // data for that type was read
  bool present[2] = {false, false};
  MGData mg[2];
  CEData ce[2];
};

struct Material {
  std::string name;
  double number_density = 0;
  std::vector<int32_t> nuclides;  // sorted by nuclide creation number
  std::vector<double> afrac;      // normalized to unit sum
  std::vector<double> afrac_raw;  // as given in the input
};

// Bins (src/Bins.cpp): none, linspace, logspace or explicit boundaries.
struct Bins1D {
  int32_t kind = kNoBins;
  uint64_t n_bins = 1;  // size(); for lin/log this includes the two infinite bins
  double lower = 0, upper = 0, width = 0;        // linspace
  double base = 10, log_lower = 0, log_upper = 0, log_width = 0;  // logspace
  std::vector<double> boundaries;
  uint64_t size() const { return kind == kBoundaries ? boundaries.size() + 1 : n_bins; }
  uint64_t index(double v) const;
};

struct Estimator {
  std::string name;
  int32_t kind = kCurrent;
  int32_t surface = -1;  // current
  int32_t cell = -1;     // track length (extension)
  bool has_cosine = false;
  double cosine_dir[3] = {1, 0, 0};
  Bins1D cosine, energy;
  // Sensitivity estimators (src/Estimator.cpp:76-90): perturbation indices
  // in the order of the `sensitivities` node; each shares the estimator's
  // bins (src/Scorable.cpp:22-29)
  std::vector<int32_t> sensitivities;
  uint64_t stride() const { return energy.size(); }
  uint64_t size() const { return cosine.size() * energy.size(); }
  // flattened bins of the estimator followed by those of its sensitivities
  uint64_t span() const { return size() * (1 + sensitivities.size()); }
};

// TotalCrossSectionPerturbation (src/Perturbation.cpp:43-83): a change in
// one nuclide's total cross section
struct Perturbation {
  std::string name;
  int32_t nuclide = -1;
};

struct Source {
  double position[3] = {0, 0, 0};
  int32_t direction = kDirIsotropic;
  double dir[3] = {1, 0, 0};  // constant direction or isotropic-flux reference
  double energy = 0;          // continuous energy (MeV)
  uint64_t group = 1;         // multigroup group
  int32_t type = kNeutron;
};

struct Model {
  // general
  std::vector<int32_t> particle_types;
  uint64_t histories = 0;
  uint64_t threads = 1;
  uint64_t chunksize = 0;
  uint64_t seed = 1;
  int32_t tracking = kSurfaceTracking;
  // problem
  int32_t problem = kFixedSource;
  uint64_t inactive = 0, active = 0;
  Source source;
  // physics
  int32_t energy_mode = kMultigroup;
  uint64_t groups = 0;
  std::vector<Surface> surfaces;
  std::vector<Nuclide> nuclides;
  std::vector<Material> materials;
  std::vector<ScalarField> fields;  // fields[0] is the global temperature field
  std::vector<Cell> cells;
  std::vector<TSLData> tsl;
  std::vector<Estimator> estimators;
  std::vector<Perturbation> perturbations;

  bool HasConstantTemperature() const { return fields[0].IsConstant(); }
  size_t total_bins() const;
};

// Loads a problem.  Relative data-file paths resolve against base_dir (the
// directory of the XML file) when it is non-empty.  Throws
// std::runtime_error with the reference's message text where the reference
// has one.
Model load_model(const std::string& xml_text, const std::string& base_dir);

// Reads a project table file (.mctab) holding one pandas-style MultiIndex
// table: the level axes and the flattened values in row-major order with
// level 0 slowest (the layout src/HDF5DataSet.hpp:132-148 indexes).
struct TableFile {
  std::vector<std::vector<double>> axes;
  std::vector<double> values;
};
TableFile read_table_file(const std::string& path);

}  // namespace mc

// XML -> flat problem model (see mc_model.hpp).
#include "mc_model.hpp"

#include "mc_xml.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <map>
#include <numeric>
#include <sstream>
#include <stdexcept>

namespace mc {

namespace {

using mcxml::Node;

constexpr double kRoomTemperature = 293.6;            // src/Constants.hpp:22
constexpr double kRelativeTemperatureTolerance = 0.01;  // src/Constants.hpp:29

std::string attr(const Node* n, const char* name, const std::string& def = "") {
  if (!n) return def;
  const std::string* a = n->attribute(name);
  return a ? *a : def;
}

bool has_attr(const Node* n, const char* name) { return n && n->attribute(name); }

// pugixml's as_double: strtod on the attribute, default when absent
double attr_double(const Node* n, const char* name, double def = 0) {
  const std::string* a = n ? n->attribute(name) : nullptr;
  if (!a) return def;
  return std::strtod(a->c_str(), nullptr);
}

uint64_t attr_u64(const Node* n, const char* name, uint64_t def = 0) {
  const std::string* a = n ? n->attribute(name) : nullptr;
  if (!a) return def;
  return std::strtoull(a->c_str(), nullptr, 10);
}

const Node* child(const Node* n, const char* name) { return n ? n->child(name) : nullptr; }

const Node* first_element(const Node* n) {
  if (!n) return nullptr;
  for (const auto& c : n->children)
    if (c->kind == Node::Kind::element) return c.get();
  return nullptr;
}

const Node* find_by_attr(const Node* parent, const char* a, const std::string& v) {
  if (!parent) return nullptr;
  for (const Node* c : parent->elements())
    if (attr(c, a) == v) return c;
  return nullptr;
}

std::string name_list(const Node* parent) {
  std::string out;
  if (!parent) return out;
  for (const Node* c : parent->elements()) out += "\"" + attr(c, "name") + "\", ";
  return out;
}

std::string resolve(const std::string& base_dir, const std::string& p) {
  if (p.empty() || p[0] == '/' || base_dir.empty()) return p;
  return base_dir + "/" + p;
}

std::vector<double> parse_reals(const std::string& s) {
  std::vector<double> out;
  std::stringstream ss{s};
  double v;
  while (ss >> v) out.push_back(v);
  return out;
}

// HDF5DataSet<D> + ToContinuousMap (src/HDF5DataSet.hpp:41-60, :87-130): a
// one-level table becomes a sorted map from axis value to value.
TableFile read_levels(const std::string& path, size_t levels) {
  TableFile t = read_table_file(path);
  if (t.axes.size() != levels) {
    throw std::runtime_error(
        path + ": Expected " + std::to_string(levels) + " dimensions, but got " + std::to_string(t.axes.size()));
  }
  return t;
}

Table1D read_map(const std::string& path) {
  TableFile t = read_levels(path, 1);
  std::map<double, double> m;
  for (size_t i = 0; i < t.axes[0].size(); i++) m[t.axes[0][i]] = t.values.at(i);
  Table1D out;
  for (const auto& [k, v] : m) {
    out.x.push_back(k);
    out.y.push_back(v);
  }
  return out;
}

// Multigroup::OneDimensional(groupxs_node) (src/Multigroup.cpp:86-99)
std::vector<double> read_group_xs(const Node* n, uint64_t G) {
  auto v = parse_reals(n->child_value());
  if (v.size() != G) {
    throw std::runtime_error(
        n->path() + ": Expected " + std::to_string(G) + " entries but got " + std::to_string(v.size()));
  }
  return v;
}

// Multigroup::TwoDimensional (src/Multigroup.cpp:124-147): XML rows are
// outgoing groups, columns incoming groups.  Returned by incoming group.
std::vector<double> read_group_matrix(const Node* n, uint64_t G, bool normalize) {
  auto flat = parse_reals(n->child_value());
  if (flat.size() != G * G) {
    throw std::runtime_error(
        n->path() + ": Expected " + std::to_string(G * G) + " entries but got " + std::to_string(flat.size()));
  }
  std::vector<double> m(G * G);
  for (uint64_t gp = 0; gp < G; gp++) {
    for (uint64_t g = 0; g < G; g++) m[gp * G + g] = flat[G * g + gp];
    if (normalize) {
      // NormalizedTwoDimensional (src/Multigroup.cpp:168-186): sum then divide
      double sum = 0;
      for (uint64_t g = 0; g < G; g++) sum += m[gp * G + g];
      if (sum != 0.)
        for (uint64_t g = 0; g < G; g++) m[gp * G + g] = m[gp * G + g] / sum;
    }
  }
  return m;
}

int reaction_kind(const std::string& name) {
  // ToReaction (src/Reaction.cpp:6-19)
  if (name == "capture") return kCapture;
  if (name == "scatter") return kScatter;
  if (name == "fission") return kFission;
  throw std::runtime_error("Unrecognized reaction name: " + name);
}

MGData read_mg(const Node* particle_node, uint64_t G) {
  MGData d;
  // member construction order of Multigroup (src/Multigroup.hpp:117-128):
  // nubar, chi, scatter_probs, reactions, total
  const Node* fission = particle_node->child("fission");
  if (const Node* nb = child(fission, "nubar")) d.nubar = read_group_xs(nb, G);
  if (const Node* chi = child(fission, "chi")) d.chi = read_group_matrix(chi, G, true);
  if (const Node* sc = particle_node->child("scatter")) d.scatter_prob = read_group_matrix(sc, G, true);
  d.total.assign(G, 0.0);
  // reactions are kept in a std::map keyed by Reaction, so the summation
  // order for the total is capture, scatter, fission (src/Multigroup.cpp:231-243)
  std::map<int, std::vector<double>> reactions;
  for (const Node* r : particle_node->elements()) {
    const int kind = reaction_kind(r->name);
    std::vector<double> xs;
    if (kind == kScatter) {
      // column sums of the (unnormalized) matrix (src/Multigroup.cpp:201-210)
      auto m = read_group_matrix(r, G, false);
      xs.assign(G, 0.0);
      for (uint64_t gp = 0; gp < G; gp++) {
        double s = 0;
        for (uint64_t g = 0; g < G; g++) s += m[gp * G + g];
        xs[gp] = s;
      }
    }
    else if (kind == kFission) {
      const Node* x = r->child("xs");
      if (!x) throw std::runtime_error(r->path() + ": \"xs\" node not found");
      xs = read_group_xs(x, G);
    }
    else {
      xs = read_group_xs(r, G);
    }
    reactions.emplace(kind, xs);  // first occurrence wins, as std::map::emplace
  }
  for (const auto& [kind, xs] : reactions) {
    for (uint64_t g = 0; g < G; g++) d.total[g] = d.total[g] + xs[g];
    if (kind == kCapture) { d.has_capture = true; d.capture = xs; }
    if (kind == kScatter) { d.has_scatter = true; d.scatter = xs; }
    if (kind == kFission) { d.has_fission = true; d.fission = xs; }
  }
  if (d.has_scatter && d.scatter_prob.empty()) throw std::runtime_error(particle_node->path() + ": scatter matrix missing");
  if (d.has_fission && (d.nubar.empty() || d.chi.empty()))
    throw std::runtime_error(particle_node->path() + "/fission: nubar and chi are required");
  return d;
}

CEEval read_eval(const Node* n, const std::string& base) {
  CEEval e;
  e.xs = read_map(resolve(base, attr(n, "file")));
  e.temperature = attr_double(n, "temperature");
  return e;
}

void read_pod_partitions(const Node* parts, const char* grid_attr, const std::string& base, PODPartitionSet& out) {
  for (const Node* p : parts ? parts->elements() : std::vector<const Node*>{}) {
    TableFile cdf = read_levels(resolve(base, attr(p, "CDF")), 2);
    TableFile s = read_levels(resolve(base, attr(p, "S")), 1);
    TableFile gt = read_levels(resolve(base, attr(p, grid_attr)), 3);
    out.F.push_back(cdf.axes[0]);
    out.cdf_modes.push_back(cdf.values);
    out.S.push_back(s.values);
    out.grid.push_back(gt.axes[0]);
    out.T.push_back(gt.axes[1]);
    out.g_t_modes.push_back(gt.values);
    out.concat.insert(out.concat.end(), gt.axes[0].begin(), gt.axes[0].end());
    out.ends.push_back(out.concat.size());
    if (cdf.axes[1].size() != s.axes[0].size() || gt.axes[2].size() != s.axes[0].size())
      throw std::runtime_error(p->path() + ": POD rank mismatch between CDF, S and mode tables");
  }
  for (size_t i = 1; i < out.concat.size(); i++)
    if (!(out.concat[i - 1] < out.concat[i]))
      throw std::runtime_error("thermal scattering partitions are not monotonically increasing");
}

TSLData read_tsl(const Node* tsl_node, const std::string& base) {
  TSLData t;
  t.majorant = read_map(resolve(base, attr(tsl_node, "majorant")));
  TableFile T = read_levels(resolve(base, attr(tsl_node, "total_T")), 2);
  TableFile S = read_levels(resolve(base, attr(tsl_node, "total_S")), 1);
  TableFile E = read_levels(resolve(base, attr(tsl_node, "total_E")), 2);
  t.xs_T = T.axes[0];
  t.xs_T_modes = T.values;
  t.xs_S = S.values;
  t.xs_E = E.axes[0];
  t.xs_E_modes = E.values;
  t.xs_rank = S.values.size();
  read_pod_partitions(tsl_node->child("beta_partitions"), "E_T", base, t.beta);
  read_pod_partitions(tsl_node->child("alpha_partitions"), "beta_T", base, t.alpha);
  t.beta_cutoff = attr_double(tsl_node, "beta_cutoff");
  t.alpha_cutoff = attr_double(tsl_node, "alpha_cutoff");
  return t;
}

CEData read_ce(const Node* particle_node, double awr, const std::string& base, std::vector<TSLData>& tsl, int type) {
  CEData d;
  d.awr = awr;
  for (const Node* r : particle_node->elements()) {
    if (r->name == "total") continue;
    CEReaction cr;
    cr.kind = reaction_kind(r->name);
    if (cr.kind == kCapture) {
      cr.eval = read_eval(r, base);
    }
    else if (cr.kind == kScatter) {
      cr.eval = read_eval(r->child("xs"), base);
      if (const Node* ts = r->child("tsl")) {
        if (type != kNeutron)
          throw std::runtime_error(ts->path() + ": Only neutrons may have a thermal scattering library node");
        tsl.push_back(read_tsl(ts, base));
        tsl.back().awr = awr;
        cr.tsl = static_cast<int32_t>(tsl.size() - 1);
      }
    }
    else {
      cr.eval = read_eval(r->child("xs"), base);
      if (const Node* nb = r->child("nubar")) {
        cr.has_nubar = true;
        cr.nubar = read_map(resolve(base, attr(nb, "file")));
      }
    }
    d.reactions.push_back(std::move(cr));
  }
  const Node* total = particle_node->child("total");
  if (!total) throw std::runtime_error(particle_node->path() + ": \"total\" node not found");
  d.total = read_eval(total, base);
  return d;
}

Bins1D read_bins(const Node* bins_node) {
  Bins1D b;
  if (!bins_node) return b;
  const std::string kind = bins_node->name;
  if (kind == "linspace") {
    b.kind = kLinspace;
    b.n_bins = attr_u64(bins_node, "bins") + 2;
    b.lower = attr_double(bins_node, "min");
    b.upper = attr_double(bins_node, "max");
    if (b.upper <= b.lower) throw std::runtime_error(bins_node->path() + ": max must be strictly greater than min");
    b.width = (b.upper - b.lower) / static_cast<double>(b.n_bins - 2);
  }
  else if (kind == "logspace") {
    b.kind = kLogspace;
    b.n_bins = attr_u64(bins_node, "bins") + 2;
    b.base = attr_double(bins_node, "base", 10);
    b.log_lower = attr_double(bins_node, "min");
    b.log_upper = attr_double(bins_node, "max");
    if (b.log_upper <= b.log_lower) throw std::runtime_error(bins_node->path() + ": max must be strictly greater than min");
    b.log_width = (b.log_upper - b.log_lower) / static_cast<double>(b.n_bins - 2);
  }
  else if (kind == "boundaries") {
    b.kind = kBoundaries;
    double prev = -INFINITY;
    for (double v : parse_reals(bins_node->child_value())) {
      if (v <= prev)
        throw std::runtime_error(
            bins_node->path() + ": nonincreasing elements found: " + std::to_string(prev) + " " + std::to_string(v));
      b.boundaries.push_back(v);
      prev = v;
    }
    b.n_bins = b.boundaries.size() + 1;
  }
  else {
    throw std::runtime_error(bins_node->path() + ": unknown bins type");
  }
  return b;
}

ScalarField read_field(const Node* n) {
  // ScalarField::Create (src/ScalarField.cpp:13-27)
  ScalarField f;
  if (!n) throw std::runtime_error("temperature: missing scalar field");
  if (n->name == "constant") {
    f.c = attr_double(n, "c");
    f.upper = f.lower = f.c;
  }
  else if (n->name == "linear") {
    f.linear = 1;
    f.upper = attr_double(child(n, "bounds"), "upper");
    f.lower = attr_double(child(n, "bounds"), "lower");
    const Node* g = child(n, "gradient");
    f.g[0] = attr_double(g, "x");
    f.g[1] = attr_double(g, "y");
    f.g[2] = attr_double(g, "z");
    f.b = attr_double(child(n, "intercept"), "b");
  }
  else {
    throw std::runtime_error(n->path() + ": unknown scalar field type");
  }
  return f;
}

Surface read_surface(const Node* surfaces, const std::string& name) {
  const Node* s = find_by_attr(surfaces, "name", name);
  if (!s) {
    throw std::runtime_error(
        "Surface node \"" + name + "\" not found. Must be one of: [" + name_list(surfaces) + "]");
  }
  Surface out;
  out.name = name;
  const std::string r = attr(s, "reflective", attr(s, "boundary"));
  out.reflective = (r == "true" || r == "1" || r == "reflective") ? 1 : 0;
  if (s->name == "sphere") {
    out.kind = kSphere;
    const Node* c = child(s, "center");
    out.p[0] = attr_double(c, "x");
    out.p[1] = attr_double(c, "y");
    out.p[2] = attr_double(c, "z");
    out.p[3] = attr_double(child(s, "radius"), "r");
  }
  else if (s->name == "planex") { out.kind = kPlaneX; out.p[0] = attr_double(s, "x"); }
  else if (s->name == "planey") { out.kind = kPlaneY; out.p[0] = attr_double(s, "y"); }
  else if (s->name == "planez") { out.kind = kPlaneZ; out.p[0] = attr_double(s, "z"); }
  else if (s->name == "cylinderx") { out.kind = kCylinderX; out.p[0] = attr_double(s, "r"); }
  else if (s->name == "cylindery") { out.kind = kCylinderY; out.p[0] = attr_double(s, "r"); }
  else if (s->name == "cylinderz") { out.kind = kCylinderZ; out.p[0] = attr_double(s, "r"); }
  else throw std::runtime_error(s->path() + ": unknown surface type");
  if (out.reflective && out.kind != kPlaneX && out.kind != kPlaneY && out.kind != kPlaneZ)
    throw std::runtime_error(s->path() + ": reflective boundaries are supported on planes only");
  return out;
}

void normalize3(double d[3]) {
  // Point::Normalize (src/Point.cpp:46-49): divide by sqrt(d.d)
  const double n = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  d[0] /= n;
  d[1] /= n;
  d[2] /= n;
}

Source read_source(const Node* src, int energy_mode) {
  Source s;
  const Node* pos = first_element(child(src, "position"));
  if (!pos || pos->name != "constant") throw std::runtime_error("source: only constant positions are supported");
  s.position[0] = attr_double(pos, "x");
  s.position[1] = attr_double(pos, "y");
  s.position[2] = attr_double(pos, "z");
  const Node* dir = first_element(child(src, "direction"));
  if (!dir) throw std::runtime_error("source: direction distribution missing");
  if (dir->name == "constant") s.direction = kDirConstant;
  else if (dir->name == "isotropic") s.direction = kDirIsotropic;
  else if (dir->name == "isotropic-flux") s.direction = kDirIsotropicFlux;
  else throw std::runtime_error(dir->path() + ": unknown direction distribution");
  if (s.direction != kDirIsotropic) {
    s.dir[0] = attr_double(dir, "x");
    s.dir[1] = attr_double(dir, "y");
    s.dir[2] = attr_double(dir, "z");
    normalize3(s.dir);
  }
  const Node* en = first_element(child(src, "energy"));
  if (!en || en->name != "constant") throw std::runtime_error("source: only constant energies are supported");
  const std::string ev = attr(en, "energy");
  if (energy_mode == kMultigroup) s.group = std::stoull(ev);
  else s.energy = std::stod(ev);
  const Node* pt = first_element(child(src, "particletype"));
  const std::string t = attr(pt, "type", "neutron");
  s.type = t == "photon" ? kPhoton : kNeutron;
  return s;
}

}  // namespace

bool CEEval::IsValid(double requested) const {
  // signed relative error, src/ContinuousEvaluation.cpp:17-20
  const double relative_error = (requested - temperature) / temperature;
  return relative_error < kRelativeTemperatureTolerance;
}

uint64_t Bins1D::index(double v) const {
  switch (kind) {
  case kLinspace:
    if (v < lower) return 0;
    if (v >= upper) return n_bins - 1;
    return static_cast<uint64_t>((v - lower) / width + 1);
  case kLogspace: {
    const double log_v = std::log(v) / std::log(base);
    if (log_v < log_lower) return 0;
    if (log_v >= log_upper) return n_bins - 1;
    return static_cast<uint64_t>((log_v - log_lower) / log_width + 1);
  }
  case kBoundaries:
    return static_cast<uint64_t>(std::upper_bound(boundaries.begin(), boundaries.end(), v) - boundaries.begin());
  default:
    return 0;
  }
}

size_t Model::total_bins() const {
  size_t n = 0;
  for (const auto& e : estimators) n += e.span();
  return n;
}

TableFile read_table_file(const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw std::runtime_error("File not found: " + path);
  char magic[8];
  in.read(magic, 8);
  if (!in || std::memcmp(magic, "MCTAB1\0\0", 8) != 0) throw std::runtime_error(path + ": not a table file");
  auto read_u64 = [&]() {
    uint64_t v = 0;
    in.read(reinterpret_cast<char*>(&v), 8);
    if (!in) throw std::runtime_error(path + ": truncated table file");
    return v;
  };
  auto read_vec = [&](uint64_t n) {
    std::vector<double> v(n);
    in.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(n * 8));
    if (!in) throw std::runtime_error(path + ": truncated table file");
    return v;
  };
  TableFile t;
  const uint64_t levels = read_u64();
  if (levels == 0 || levels > 8) throw std::runtime_error(path + ": bad level count");
  uint64_t expect = 1;
  for (uint64_t l = 0; l < levels; l++) {
    const uint64_t n = read_u64();
    t.axes.push_back(read_vec(n));
    expect *= n;
  }
  const uint64_t nv = read_u64();
  if (nv != expect) throw std::runtime_error(path + ": value count does not match axes");
  t.values = read_vec(nv);
  return t;
}

Model load_model(const std::string& xml_text, const std::string& base_dir) {
  auto doc = mcxml::parse(xml_text);
  const Node* root = doc->child("minimc");
  if (!root) throw std::runtime_error("root element <minimc> not found");
  Model m;

  // general (src/Driver.cpp:37-52, src/minimc.xsd:9-20)
  const Node* general = child(root, "general");
  if (!general) throw std::runtime_error("/minimc/general not found");
  {
    std::stringstream ss{general->child("particles") ? general->child("particles")->child_value() : ""};
    std::string p;
    while (ss >> p) {
      if (p == "neutron") m.particle_types.push_back(kNeutron);
      else if (p == "photon") m.particle_types.push_back(kPhoton);
      else throw std::runtime_error("/minimc/general/particles: unknown particle type " + p);
    }
    if (m.particle_types.empty()) throw std::runtime_error("/minimc/general/particles: empty");
  }
  auto req = [&](const char* name) -> std::string {
    const Node* n = general->child(name);
    if (!n) throw std::runtime_error(std::string("/minimc/general/") + name + " not found");
    return n->child_value();
  };
  m.histories = static_cast<uint64_t>(std::stoll(req("histories")));
  m.threads = std::stoul(req("threads"));
  if (const Node* c = general->child("chunksize")) m.chunksize = std::stoull(c->child_value());
  m.seed = general->child("seed") ? static_cast<uint64_t>(std::stoll(general->child("seed")->child_value())) : 1;
  const std::string tracking = general->child("tracking") ? general->child("tracking")->child_value() : "";

  // nuclear data kind
  const Node* nuclides_node = child(root, "nuclides");
  const Node* energy_node = first_element(nuclides_node);
  if (!energy_node) throw std::runtime_error("/minimc/nuclides is empty");
  if (energy_node->name == "multigroup") {
    m.energy_mode = kMultigroup;
    m.groups = attr_u64(energy_node, "groups");
    if (m.groups == 0) throw std::runtime_error(energy_node->path() + ": groups must be positive");
  }
  else if (energy_node->name == "continuous") {
    m.energy_mode = kContinuous;
  }
  else {
    throw std::runtime_error(energy_node->path() + ": unknown nuclear data type");
  }

  const Node* surfaces_node = child(root, "surfaces");
  const Node* materials_node = child(root, "materials");
  const Node* cells_node = child(root, "cells");
  if (!cells_node) throw std::runtime_error("/minimc/cells not found");
  const auto cell_nodes = cells_node->elements();

  // surfaces in order of first appearance (src/World.cpp:98-115)
  std::map<std::string, int32_t> surface_index;
  for (const Node* c : cell_nodes) {
    for (const Node* s : c->elements()) {
      const std::string n = attr(s, "name");
      if (surface_index.count(n)) continue;
      m.surfaces.push_back(read_surface(surfaces_node, n));
      surface_index[n] = static_cast<int32_t>(m.surfaces.size() - 1);
    }
  }

  auto find_material_node = [&](const std::string& name) {
    // Material::FindNode (src/Material.cpp:14-30)
    const Node* mn = find_by_attr(materials_node, "name", name);
    if (!mn) {
      throw std::runtime_error(
          "Material node \"" + name + "\" not found. Must be one of: [" + name_list(materials_node) + "]");
    }
    return mn;
  };

  // nuclides in order of first appearance (src/World.cpp:117-160)
  std::map<std::string, int32_t> nuclide_index;
  for (const Node* c : cell_nodes) {
    if (c->name == "void") continue;
    const Node* mn = find_material_node(attr(c, "material"));
    for (const Node* mnuc : mn->elements()) {
      const std::string nn = attr(mnuc, "name");
      if (nuclide_index.count(nn)) continue;
      const Node* nn_node = find_by_attr(energy_node, "name", nn);
      if (!nn_node) {
        throw std::runtime_error(
            "Nuclide node \"" + nn + "\" not found. Must be one of: [" + name_list(energy_node) + "]");
      }
      Nuclide nuc;
      nuc.name = nn;
      // Interaction::Create (src/Interaction.cpp:16-46)
      for (int32_t t : m.particle_types) {
        const char* tname = t == kNeutron ? "neutron" : "photon";
        const Node* pn = nn_node->child(tname);
        if (!pn) throw std::runtime_error(nn_node->path() + ": \"" + tname + "\" node not found");
        nuc.present[t] = true;
        if (m.energy_mode == kMultigroup) nuc.mg[t] = read_mg(pn, m.groups);
        else nuc.ce[t] = read_ce(pn, attr_double(nn_node, "awr"), base_dir, m.tsl, t);
      }
      m.nuclides.push_back(std::move(nuc));
      nuclide_index[nn] = static_cast<int32_t>(m.nuclides.size() - 1);
    }
  }

  // materials in order of first appearance (src/World.cpp:162-184)
  std::map<std::string, int32_t> material_index;
  for (const Node* c : cell_nodes) {
    if (c->name == "void") continue;
    const std::string name = attr(c, "material");
    if (material_index.count(name)) continue;
    const Node* mn = find_material_node(name);
    Material mat;
    mat.name = name;
    mat.number_density = attr_double(mn, "aden");
    std::vector<std::pair<int32_t, double>> fr;
    for (const Node* mnuc : mn->elements()) {
      const int32_t idx = nuclide_index.at(attr(mnuc, "name"));
      bool dup = false;
      for (auto& f : fr) dup = dup || f.first == idx;
      if (!dup) fr.emplace_back(idx, attr_double(mnuc, "afrac"));
    }
    std::sort(fr.begin(), fr.end());
    // normalization (src/Material.cpp:80-93): sum in map order, then divide
    double sum = 0;
    for (auto& f : fr) sum += f.second;
    for (auto& f : fr) {
      mat.nuclides.push_back(f.first);
      mat.afrac.push_back(f.second / sum);
      mat.afrac_raw.push_back(f.second);
    }
    m.materials.push_back(std::move(mat));
    material_index[name] = static_cast<int32_t>(m.materials.size() - 1);
  }

  // temperature (src/World.cpp:186-193)
  if (const Node* t = child(root, "temperature")) m.fields.push_back(read_field(first_element(t)));
  else {
    ScalarField f;
    f.c = f.upper = f.lower = kRoomTemperature;
    m.fields.push_back(f);
  }

  // cells (src/Cell.cpp:17-23, :55-113)
  for (const Node* c : cell_nodes) {
    Cell cell;
    cell.name = attr(c, "name");
    if (c->name != "void" && c->name != "cell") throw std::runtime_error(c->path() + ": unknown cell type");
    std::vector<std::pair<int32_t, uint8_t>> ss;
    for (const Node* s : c->elements()) {
      const int32_t idx = surface_index.at(attr(s, "name"));
      const std::string sense = attr(s, "sense");
      uint8_t within;
      if (sense == "-1") within = 1;
      else if (sense == "+1") within = 0;
      else throw std::runtime_error(s->path() + ": sense must be \"-1\" or \"+1\"");
      bool dup = false;
      for (auto& p : ss) dup = dup || p.first == idx;
      if (!dup) ss.emplace_back(idx, within);
    }
    std::sort(ss.begin(), ss.end());
    for (auto& p : ss) {
      cell.surfaces.push_back(p.first);
      cell.within.push_back(p.second);
    }
    // AssignMaterial: a node without a name attribute is a void
    cell.material = has_attr(c, "name") && c->name != "void" ? material_index.at(attr(c, "material")) : -1;
    if (has_attr(c, "temperature")) {
      ScalarField f;
      f.c = f.upper = f.lower = attr_double(c, "temperature");
      m.fields.push_back(f);
      cell.temperature = static_cast<int32_t>(m.fields.size() - 1);
    }
    else {
      cell.temperature = 0;
    }
    m.cells.push_back(std::move(cell));
  }

  // tracking (src/TransportMethod.cpp:23-46)
  if (tracking.empty() || tracking == "surface") {
    if (!m.HasConstantTemperature())
      throw std::runtime_error("Surface tracking with continuous global temperature not allowed");
    m.tracking = kSurfaceTracking;
  }
  else if (tracking == "cell delta") {
    m.tracking = kCellDeltaTracking;
  }
  else {
    throw std::runtime_error("/minimc/general/tracking: unknown tracking type " + tracking);
  }

  // problem type and source (src/Driver.cpp:18-35, src/KEigenvalue.cpp:19-34)
  const Node* pt = first_element(child(root, "problemtype"));
  if (!pt) throw std::runtime_error("/minimc/problemtype is empty");
  if (pt->name == "fixedsource") {
    m.problem = kFixedSource;
    m.source = read_source(pt, m.energy_mode);
  }
  else if (pt->name == "keigenvalue") {
    m.problem = kKEigenvalue;
    m.inactive = attr_u64(pt, "inactive");
    m.active = attr_u64(pt, "active");
    m.source = read_source(pt->child("initialsource"), m.energy_mode);
  }
  else {
    throw std::runtime_error(pt->path() + ": unknown problem type");
  }
  if (m.energy_mode == kMultigroup && (m.source.group < 1 || m.source.group > m.groups))
    throw std::runtime_error("source group out of range");

  // perturbations (src/Driver.cpp:38, src/Perturbation.cpp:22-50, 87-96)
  if (const Node* ps = child(root, "perturbations")) {
    for (const Node* pn : ps->elements()) {
      if (pn->name != "total") throw std::runtime_error(pn->path() + ": unknown perturbation type");
      Perturbation pert;
      pert.name = attr(pn, "name");
      const std::string nn = attr(pn, "nuclide");
      auto it = nuclide_index.find(nn);
      if (it == nuclide_index.end()) {
        // World::FindNuclideByName (src/World.cpp:63-81)
        std::string names;
        for (const auto& n : m.nuclides) names += "\"" + n.name + "\", ";
        throw std::runtime_error("Nuclide \"" + nn + "\" not found. Must be one of: [" + names + "]");
      }
      pert.nuclide = it->second;
      m.perturbations.push_back(std::move(pert));
    }
  }

  // estimators (src/Estimator.cpp:21-33, :185-205)
  if (const Node* es = child(root, "estimators")) {
    for (const Node* e : es->elements()) {
      Estimator est;
      est.name = attr(e, "name");
      if (e->name == "current") {
        est.kind = kCurrent;
        const std::string sname = attr(e, "surface");
        auto it = surface_index.find(sname);
        if (it == surface_index.end()) {
          // World::FindSurfaceByName (src/World.cpp:43-62)
          std::string names;
          for (const auto& s : m.surfaces) names += "\"" + s.name + "\", ";
          throw std::runtime_error("Surface \"" + sname + "\" not found. Must be one of: [" + names + "]");
        }
        est.surface = it->second;
      }
      else if (e->name == "tracklength") {
        est.kind = kTrackLength;
        const std::string cname = attr(e, "cell");
        for (size_t i = 0; i < m.cells.size(); i++)
          if (m.cells[i].name == cname && m.cells[i].material >= 0) est.cell = static_cast<int32_t>(i);
        if (est.cell < 0) throw std::runtime_error("Cell \"" + cname + "\" not found for track-length estimator");
      }
      else {
        throw std::runtime_error(e->path() + ": unknown estimator type");
      }
      const Node* bins = e->child("bins");
      const Node* cosine = child(bins, "cosine");
      if (cosine) {
        est.has_cosine = true;
        est.cosine_dir[0] = attr_double(cosine, "u");
        est.cosine_dir[1] = attr_double(cosine, "v");
        est.cosine_dir[2] = attr_double(cosine, "w");
        normalize3(est.cosine_dir);
      }
      est.cosine = read_bins(first_element(cosine));
      est.energy = read_bins(first_element(child(bins, "energy")));
      if (const Node* sn = e->child("sensitivities")) {
        for (const Node* sp : sn->elements()) {
          // Sensitivity::Create (src/Sensitivity.cpp:13-21): the perturbation
          // by name, then TotalCrossSectionPerturbation::CreateSensitivity
          // (src/Perturbation.cpp:52-66), which supports current estimators
          const std::string pname = attr(sp, "name");
          int32_t k = -1;
          for (size_t i = 0; i < m.perturbations.size(); i++)
            if (m.perturbations[i].name == pname) k = static_cast<int32_t>(i);
          if (k < 0) {
            // PerturbationSet::FindPerturbationByName (src/Perturbation.cpp:98-118)
            std::string names;
            for (const auto& q : m.perturbations) names += "\"" + q.name + "\", ";
            throw std::runtime_error("Perturbation \"" + pname + "\" not found. Must be one of: [" + names + "]");
          }
          if (est.kind != kCurrent)
            throw std::runtime_error(
                "Sensitivity to total cross section perturbation not supported for estimator: " + e->path());
          est.sensitivities.push_back(k);
        }
      }
      m.estimators.push_back(std::move(est));
    }
  }
  return m;
}

}  // namespace mc

// simulation.cpp -- Simulation: scene -> engine plan -> GPU step loop.
//
// Simulation::init performs what the reference's init() does
// (src/simulation/simulation_init.cpp:10-22) but produces the compact plan of
// include/xfdtd_cuda.h instead of 18 per-cell coefficient arrays:
//
//   grid space            simulation_init.cpp:105-146, grid_space.cpp:351-638
//   dt                    fdtd_basic_coff.cpp:11-29, 342-346
//   object rasterisation  object.cpp:53-73 (cell centre test, last writer wins)
//   coefficients          fdtd_basic_coff.cpp:77-121 -> one table entry per
//                         distinct (material, override) tuple
//   thin wires            thin_wire.cpp:39-129 (coefficient overrides)
//   lumped elements       current_source.cpp, voltage_source.cpp,
//                         resistor.cpp, capacitor.cpp, inductor.cpp
//   CPML                  perfect_match_layer.cpp:133-432 -> 1-D profiles
//   TFSF                  tfsf.cpp:15-53, tfsf_3d.cpp:13-151
//   NF-FF                 nffft.cpp:22-34, nffft_fd.cpp:17-106
//   monitors              voltage_monitor.cpp:25-62, current_monitor.cpp:23-68
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../../include/xfdtd_cuda.h"
#include "xfdtd/xfdtd.h"

namespace xfdtd {

namespace {

// f(q) for q in [0, n), split over the host's cores in contiguous chunks;
// every q is independent (rasterisation and index raster: one cell or one
// plane each).
template <typename F>
void parallel_for(size_t n, F &&f) {
  const size_t hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::min<size_t>(std::min<size_t>(hw, 64), n);
  if (nt <= 1) {
    for (size_t q = 0; q < n; ++q) f(q);
    return;
  }
  std::vector<std::thread> pool;
  const size_t per = (n + nt - 1) / nt;
  for (size_t t = 0; t < nt; ++t)
    pool.emplace_back([&, t] {
      const size_t lo = t * per, hi = std::min(n, lo + per);
      for (size_t q = lo; q < hi; ++q) f(q);
    });
  for (auto &th : pool) th.join();
}

}  // namespace

void checkEngine(int status, xfdtd_handle *h) {
  if (status != XFDTD_OK)
    throw std::runtime_error(std::string("GPU engine: ") + (h ? xfdtd_last_error(h) : "no handle") +
                             " (status " + std::to_string(status) + ")");
}

Simulation::Simulation(double cell_size, float cfl) : _cell_size{cell_size}, _cfl{cfl} {}
Simulation::Simulation(double cell_size, std::vector<std::shared_ptr<Object>> objects,
                       std::vector<std::shared_ptr<Boundary>> boundaries, std::unique_ptr<TFSF> tfsf, float cfl)
    : _cell_size{cell_size}, _cfl{cfl}, _objects{std::move(objects)}, _boundaries{std::move(boundaries)},
      _tfsf{std::move(tfsf)} {}
Simulation::Simulation(double cell_size, std::vector<std::shared_ptr<Object>> objects,
                       std::vector<std::shared_ptr<Boundary>> boundaries, std::unique_ptr<TFSF> tfsf,
                       std::unique_ptr<NFFFT> nffft, float cfl)
    : _cell_size{cell_size}, _cfl{cfl}, _objects{std::move(objects)}, _boundaries{std::move(boundaries)},
      _tfsf{std::move(tfsf)}, _nffft{std::move(nffft)} {}
Simulation::Simulation(double cell_size, std::vector<std::shared_ptr<Object>> objects,
                       std::vector<std::shared_ptr<LumpedElement>> lumped_elements,
                       std::vector<std::shared_ptr<Boundary>> boundaries, std::vector<std::shared_ptr<Monitor>> monitors,
                       float cfl)
    : _cell_size{cell_size}, _cfl{cfl}, _objects{std::move(objects)}, _boundaries{std::move(boundaries)},
      _lumped_elements{std::move(lumped_elements)}, _monitors{std::move(monitors)} {}
Simulation::Simulation(double cell_size, std::vector<std::shared_ptr<Object>> objects,
                       std::vector<std::shared_ptr<Monitor>> monitors, float cfl)
    : _cell_size{cell_size}, _cfl{cfl}, _objects{std::move(objects)}, _monitors{std::move(monitors)} {}
Simulation::Simulation(double cell_size, std::vector<std::shared_ptr<Object>> objects,
                       std::vector<std::shared_ptr<LumpedElement>> lumped_elements,
                       std::vector<std::shared_ptr<Boundary>> boundaries, std::vector<std::shared_ptr<Monitor>> monitors,
                       std::unique_ptr<Network> network, float cfl)
    : _cell_size{cell_size}, _cfl{cfl}, _objects{std::move(objects)}, _boundaries{std::move(boundaries)},
      _lumped_elements{std::move(lumped_elements)}, _monitors{std::move(monitors)}, _network{std::move(network)} {}
Simulation::~Simulation() { release(); }

// util/dft.h:11-27: the phase of sample j is 2 pi f (j dt), the sum is scaled by dt
std::vector<std::complex<double>> dft(const std::vector<double> &x, double dt, const std::vector<double> &frequencies) {
  using namespace std::complex_literals;
  std::vector<std::complex<double>> r(frequencies.size());
  for (size_t q = 0; q < frequencies.size(); ++q) {
    std::complex<double> sum{0.0, 0.0};
    for (size_t j = 0; j < x.size(); ++j) {
      const double t = static_cast<double>(j) * dt;
      sum += x[j] * std::exp(-2.0 * 1i * constant::PI * frequencies[q] * t);
    }
    r[q] = sum * dt;
  }
  return r;
}

// Port::calculateSParameter, port.cpp:25-34
void Port::calculateSParameter(const std::vector<double> &frequencies, double dt) {
  const std::complex<double> z = _impedance;
  const double k = std::sqrt(std::real(z));
  const auto v = dft(_voltage->getValue(), dt, frequencies);
  const auto i = dft(_current->getValue(), dt, frequencies);
  _a.resize(v.size());
  _b.resize(v.size());
  for (size_t q = 0; q < v.size(); ++q) {
    _a[q] = 0.5 * (v[q] + z * i[q]) / k;
    _b[q] = 0.5 * (v[q] - std::conj(z) * i[q]) / k;
  }
}

// Network::outputData's arithmetic, network.cpp:40-52
void Network::calculate(double dt) {
  for (auto &p : _ports) p->calculateSParameter(_frequencies, dt);
  _s_parameters.clear();
  for (size_t i = 0; i < _ports.size(); ++i) {
    if (!_ports[i]->isActivatedSource()) continue;
    const auto &a = _ports[i]->getA();
    for (size_t j = 0; j < _ports.size(); ++j) {
      const auto &b = _ports[j]->getB();
      std::vector<std::complex<double>> s(b.size());
      for (size_t q = 0; q < b.size(); ++q) s[q] = b[q] / a[q];
      _s_parameters[_ports[j]->getPortIndex() * 10 + _ports[i]->getPortIndex()] = std::move(s);
    }
  }
}

const std::map<int, std::vector<std::complex<double>>> &Simulation::sParameters() {
  if (!_network) throw std::runtime_error("no network in this simulation");
  for (const auto &p : _network->getPorts()) {
    for (const Monitor *m : {static_cast<const Monitor *>(p->getVoltageMonitor().get()),
                             static_cast<const Monitor *>(p->getCurrentMonitor().get())}) {
      size_t q = 0;
      while (q < _monitors.size() && _monitors[q].get() != m) ++q;
      if (q == _monitors.size()) throw std::runtime_error("a port's monitor is not one of the simulation's monitors");
      _monitors[q]->setValue(monitorValues(q));
    }
  }
  _network->calculate(_dt);
  return _network->getSParameters();
}

void Simulation::release() {
  if (_engine) xfdtd_destroy(_engine);
  _engine = nullptr;
}

void Simulation::addObject(std::shared_ptr<Object> o) { _objects.push_back(std::move(o)); }
void Simulation::addBoundary(std::shared_ptr<Boundary> b) { _boundaries.push_back(std::move(b)); }
void Simulation::addLumpedElement(std::shared_ptr<LumpedElement> l) { _lumped_elements.push_back(std::move(l)); }
void Simulation::addTFSFSource(std::shared_ptr<TFSF> t) { _tfsf = std::move(t); }
void Simulation::addNFFFT(std::shared_ptr<NFFFT> n) { _nffft = std::move(n); }
void Simulation::addMonitor(std::shared_ptr<Monitor> m) { _monitors.push_back(std::move(m)); }

void Simulation::setVoxelMaterials(std::vector<Material> materials, std::vector<uint16_t> index,
                                   std::array<size_t, 3> shape) {
  setVoxelMaterials(std::move(materials), std::vector<uint32_t>(index.begin(), index.end()), shape);
}

void Simulation::setVoxelMaterials(std::vector<Material> materials, std::vector<uint32_t> index,
                                   std::array<size_t, 3> shape) {
  if (index.size() != shape[0] * shape[1] * shape[2]) throw std::invalid_argument("voxel index size mismatch");
  for (uint32_t v : index)
    if (v >= materials.size()) throw std::invalid_argument("voxel index out of range");
  _voxel_materials = std::move(materials);
  _voxel_index = std::move(index);
  _voxel_shape = shape;
}

namespace {

using Tuple = std::array<double, XFDTD_N_COEFF>;

struct Props {
  double eps, mu, se, sm;
  bool disp = false;   // a dispersive medium's cell: its E comes from the medium's recursion
  bool operator<(const Props &o) const {
    return std::tie(eps, mu, se, sm, disp) < std::tie(o.eps, o.mu, o.se, o.sm, o.disp);
  }
};

// FDTDBasicCoff::initCoff formulas (fdtd_basic_coff.cpp:77-91) for a uniform
// cell (dx, dy, dz).
Tuple coefficients(const Props &p, double dt, const double d[3]) {
  Tuple c{};
  auto e = [&](double da, double db, double &ce, double &cha, double &chb) {
    ce = (2 * p.eps - dt * p.se) / (2 * p.eps + dt * p.se);
    cha = -(2 * dt / db) / (2 * p.eps + p.se * dt);
    chb = (2 * dt / da) / (2 * p.eps + p.se * dt);
  };
  auto h = [&](double da, double db, double &ch, double &cea, double &ceb) {
    ch = (2 * p.mu - dt * p.sm) / (2 * p.mu + dt * p.sm);
    cea = (2 * dt / db) / (2 * p.mu + p.sm * dt);
    ceb = -(2 * dt / da) / (2 * p.mu + p.sm * dt);
  };
  e(d[1], d[2], c[0], c[1], c[2]);     // Ex: da = dy, db = dz
  e(d[2], d[0], c[3], c[4], c[5]);     // Ey: da = dz, db = dx
  e(d[0], d[1], c[6], c[7], c[8]);     // Ez: da = dx, db = dy
  h(d[1], d[2], c[9], c[10], c[11]);   // Hx: da = dy, db = dz
  h(d[2], d[0], c[12], c[13], c[14]);  // Hy: da = dz, db = dx
  h(d[0], d[1], c[15], c[16], c[17]);  // Hz: da = dx, db = dy
  if (p.disp)   // the volume update leaves E of a dispersive cell as it is
    for (int q = 0; q < 9; ++q) c[q] = q % 3 == 0 ? 1.0 : 0.0;
  return c;
}

// The E recursion coefficients of a linear dispersive medium, as
// LorentzMedium::init (dispersive_material.cpp:17-36), DrudeMedium::init
// (:126-142) and DebyMedium::init (:195-210) compute them.
xfdtd_dispersive_medium dispersiveMedium(const Material &m, double dt, double dl) {
  xfdtd_dispersive_medium d{};
  d.kind = m.dispersionKind();
  const auto &p = m.dispersionParams();
  const double eps_0 = constant::EPSILON_0, sigma_e = m.getElectricalConductivity();
  if (d.kind == 1) {
    const double eps_s = p[0], eps_inf = p[1], omega_p = p[2], nv = p[3];
    const double delta_eps = eps_s - eps_inf;
    const double temp_coff_0 = nv * dt + 1;
    d.alpha = (2 - omega_p * omega_p * dt * dt) / temp_coff_0;
    d.xi = (nv * dt - 1) / temp_coff_0;
    d.gamma = (eps_0 * delta_eps * omega_p * omega_p * dt * dt) / temp_coff_0;
    const double temp_coff_1 = 4 * eps_0 * eps_inf + d.gamma + 2 * sigma_e * dt;
    d.ca = (4 * eps_0 * eps_inf - 2 * sigma_e * dt) / (temp_coff_1);
    d.cb = (d.gamma) / (temp_coff_1);
    d.cc = (4 * dt) / (temp_coff_1 * dl);
  } else if (d.kind == 2) {
    const double eps_inf = p[0], omega_p = p[1], nv = p[2];
    d.k = (2 - nv * dt) / (2 + nv * dt);
    d.beta = (omega_p * omega_p * eps_0 * dt) / (2 + nv * dt);
    const double temp_coff_1 = 2 * eps_0 * eps_inf + d.beta * dt + sigma_e * dt;
    d.ca = (2 * eps_0 * eps_inf - d.beta * dt - sigma_e * dt) / (temp_coff_1);
    d.cb = 2 * dt / (temp_coff_1 * dl);
  } else if (d.kind == 3) {
    const double eps_s = p[0], eps_inf = p[1], tau = p[2];
    const double delta_eps = eps_s - eps_inf;
    d.k = (2 * tau - dt) / (2 * tau + dt);
    d.beta = (2 * delta_eps * eps_0 * dt) / (2 * tau + dt);
    const double temp_coff_1 = 2 * eps_0 * eps_inf + d.beta + sigma_e * dt;
    d.ca = (2 * eps_0 * eps_inf + d.beta - sigma_e * dt) / (temp_coff_1);
    d.cb = (2 * dt) / ((temp_coff_1)*dl);
  } else {
    throw std::runtime_error("unknown dispersive medium");
  }
  return d;
}


struct CpmlProfile {
  std::vector<int> slot_e, slot_h;
  std::vector<double> b_e, a_e, rk_e, b_m, a_m, rk_m;
  int layers = 0;
};

// Per-layer profiles of PML::initP / PML::initN (perfect_match_layer.cpp:133-155, 302-325).
void pmlLayers(const PML &p, double dl, double dt, bool positive, std::vector<double> &b_e, std::vector<double> &a_e,
               std::vector<double> &k_e, std::vector<double> &b_m, std::vector<double> &a_m, std::vector<double> &k_m) {
  const int T = p.getSize(), order = p.getOrder();
  const double e2m = constant::MU_0 / constant::EPSILON_0;
  const double sigma_max = p.getSigmaRatio() * (order + 1) / (150.0 * constant::PI * dl);
  b_e.resize(T); a_e.resize(T); k_e.resize(T); b_m.resize(T); a_m.resize(T); k_m.resize(T);
  for (int i = 0; i < T; ++i) {
    const double rho_e = positive ? (i + 1 - 0.75) / static_cast<double>(T) : (T - i - 0.75) / static_cast<double>(T);
    const double rho_m = positive ? (i + 1 - 0.25) / static_cast<double>(T) : (T - i - 0.25) / static_cast<double>(T);
    const double sigma_e = sigma_max * std::pow(rho_e, order);
    const double sigma_m = sigma_max * std::pow(rho_m, order) * e2m;
    const double kappa_e = 1 + (p.getKappaMax() - 1) * std::pow(rho_e, order);
    const double kappa_m = 1 + (p.getKappaMax() - 1) * std::pow(rho_m, order);
    const double alpha_e = p.getAlphaMin() + (p.getAlphaMax() - p.getAlphaMin()) * (1 - rho_e);
    const double alpha_m = (p.getAlphaMin() + (p.getAlphaMax() - p.getAlphaMin()) * (1 - rho_m)) * e2m;
    k_e[i] = kappa_e;
    k_m[i] = kappa_m;
    b_e[i] = std::exp((-dt / constant::EPSILON_0) * (sigma_e / kappa_e + alpha_e));
    a_e[i] = (1 / dl) * (b_e[i] - 1) * sigma_e / (kappa_e * (sigma_e + kappa_e * alpha_e));
    b_m[i] = std::exp((-dt / constant::MU_0) * (sigma_m / kappa_m + alpha_m));
    a_m[i] = (1 / dl) * (b_m[i] - 1) * sigma_m / (kappa_m * (sigma_m + kappa_m * alpha_m));
  }
}

}  // namespace

void Simulation::init(size_t total_time_steps) {
  release();
  if (total_time_steps == 0) throw std::invalid_argument("total_time_steps must be positive");
  _total = total_time_steps;

  // ---- grid space -------------------------------------------------------
  GridSpace gs(_cell_size);
  for (auto &o : _objects) {
    auto w = o->getWrappedBox();
    const Cube *c = dynamic_cast<const Cube *>(w.get());
    if (!c) throw std::runtime_error("Shape Type Error");
    gs.calculateSpaceSize(*c);
  }
  for (auto &b : _boundaries) gs.extendBoundary(b->getOrientation(), b->getSize() * gs.base(static_cast<int>(b->getOrientation()) / 2));
  gs.generateUniformGridSpace();
  _nx = gs.n(0);
  _ny = gs.n(1);
  _nz = gs.n(2);
  const size_t nx = _nx, ny = _ny, nz = _nz;
  const double d[3] = {gs.base(0), gs.base(1), gs.base(2)};
  const bool two_d = gs.dim() == 2;
  if (two_d)   // FDTDBasicCoff::init, fdtd_basic_coff.cpp:19-21: calculateDeltaT(cfl, dx, dy)
    _dt = static_cast<double>(_cfl) / (constant::C_0 * std::sqrt(1.0 / (d[0] * d[0]) + 1.0 / (d[1] * d[1])));
  else
    _dt = static_cast<double>(_cfl) / (constant::C_0 * std::sqrt(1.0 / (d[0] * d[0]) + 1.0 / (d[1] * d[1]) + 1.0 / (d[2] * d[2])));
  if (two_d && _tfsf && !dynamic_cast<const TFSF2D *>(_tfsf.get()))
    throw std::runtime_error("a 2-D grid (nz = 1) takes TFSF2D");
  if (!two_d && _tfsf && dynamic_cast<const TFSF2D *>(_tfsf.get()))
    throw std::runtime_error("TFSF2D needs a 2-D grid (nz = 1)");
  if (two_d) {
    // The 2-D path carries what the reference's 2-D example uses: objects,
    // the x and y CPML, TFSF2D and field (movie) monitors.  Its 2-D far
    // field is a debug output (nffft_broadband.cpp:173-180), and its
    // lumped elements and voltage/current monitors divide by the z cell
    // size, which a 2-D GridSpace reports as 0 (grid_space.cpp:180-186).
    if (_nffft) throw std::runtime_error("the 2-D grid (nz = 1) carries no NF-FF box");
    if (!_lumped_elements.empty()) throw std::runtime_error("the 2-D grid (nz = 1) carries no lumped elements");
    for (auto &o : _objects)
      if (o->isThinWire()) throw std::runtime_error("the 2-D grid (nz = 1) carries no thin wires");
    for (auto &m : _monitors)
      if (dynamic_cast<const VoltageMonitor *>(m.get()) || dynamic_cast<const CurrentMonitor *>(m.get()))
        throw std::runtime_error("the 2-D grid (nz = 1) carries field monitors only");
  }
  const double dt = _dt;
  if (_tfsf) _tfsf->bindTimeStep(dt);

  // ---- materials --------------------------------------------------------
  std::map<Props, uint32_t> mat_ids;
  std::vector<Props> mats;
  auto intern = [&](const Props &p) {
    auto it = mat_ids.find(p);
    if (it != mat_ids.end()) return it->second;
    uint32_t id = static_cast<uint32_t>(mats.size());
    mats.push_back(p);
    mat_ids.emplace(p, id);
    return id;
  };
  intern(Props{constant::EPSILON_0, constant::MU_0, 0.0, 0.0});   // background, fdtd_basic_coff.cpp:313-339
  std::vector<uint32_t> cell_mat(nx * ny * nz, 0);
  // dispersive media: per cell the index of its dispersive medium (-1 none)
  std::vector<xfdtd_dispersive_medium> disp_media;
  std::vector<int32_t> cell_disp;
  for (auto &o : _objects)
    if (o->isDispersion() && cell_disp.empty()) {
      // LinearDispersiveMaterial::init (dispersive_material.h:30-43)
      if (two_d || d[0] != d[1] || d[1] != d[2]) throw std::runtime_error("The condition (dx == dy == dz) is required");
      cell_disp.assign(nx * ny * nz, -1);
    }
  for (auto &o : _objects) {
    if (o->isThinWire()) {   // thin_wire.cpp:17-37: checks only
      const Cylinder *cy = dynamic_cast<const Cylinder *>(&o->shape());
      if (!cy) throw std::runtime_error("ThinWire only support Cylinder shape");
      const int ax = static_cast<int>(cy->getAxis());
      const double r = cy->getRadius();
      bool thin = true;
      for (int a = 0; a < 3; ++a)
        if (a != ax && !(r < d[a] / 2)) thin = false;
      if (!thin) throw std::runtime_error("ThinWire is not enough thin");
      continue;
    }
    gs.gridBox(o->shape());   // Object::init computes the grid box first; it throws out of range
    const Material &m = o->material();
    const uint32_t id = intern(Props{m.getPermittivityE(), m.getPermeabilityM(), m.getElectricalConductivity(),
                                     m.getMagneticConductivity(), m.isDispersion()});
    int32_t did = -1;
    if (m.isDispersion()) {
      did = static_cast<int32_t>(disp_media.size());
      disp_media.push_back(dispersiveMedium(m, dt, d[0]));
    }
    // candidate index range: cell centres within the wrapped box (plus tolerance)
    auto w = o->getWrappedBox();
    const Cube *c = dynamic_cast<const Cube *>(w.get());
    const double lo[3] = {c->getXmin(), c->getYmin(), c->getZmin()};
    const double hi[3] = {c->getXmax(), c->getYmax(), c->getZmax()};
    size_t r0[3], r1[3];
    for (int a = 0; a < 3; ++a) {
      const auto &hc = gs.hNodes(a);
      const double tol = 4 * constant::TOLERABLE_EPSILON + 1e-9 * std::abs(hi[a] - lo[a]);
      r0[a] = static_cast<size_t>(std::lower_bound(hc.begin(), hc.end(), lo[a] - tol) - hc.begin());
      r1[a] = static_cast<size_t>(std::upper_bound(hc.begin(), hc.end(), hi[a] + tol) - hc.begin());
    }
    // the 2-D mask takes the cell centre at z = 0 (GridSpace::getShapeMask
    // and getGridCenterZ, grid_space.cpp:241-247, 284-291): its one k plane
    // is a candidate whatever the z of the centre node
    if (two_d) r0[2] = 0, r1[2] = 1;
    const Shape &sh = o->shape();
    if (r1[0] > r0[0])
      parallel_for(r1[0] - r0[0], [&](size_t q) {   // planes of one object: disjoint cells
        const size_t i = r0[0] + q;
        for (size_t j = r0[1]; j < r1[1]; ++j)
          for (size_t k = r0[2]; k < r1[2]; ++k)
            if (sh.isPointInside(PointVector{gs.hNode(0, i), gs.hNode(1, j), two_d ? 0.0 : gs.hNode(2, k)})) {
              cell_mat[(i * ny + j) * nz + k] = id;
              if (!cell_disp.empty()) cell_disp[(i * ny + j) * nz + k] = did;
            }
      });
  }
  if (!_voxel_index.empty()) {
    if (_voxel_shape[0] != nx || _voxel_shape[1] != ny || _voxel_shape[2] != nz)
      throw std::runtime_error("voxel raster shape does not match the grid");
    std::vector<uint32_t> vid(_voxel_materials.size());
    for (size_t q = 0; q < vid.size(); ++q) {
      const Material &m = _voxel_materials[q];
      vid[q] = intern(Props{m.getPermittivityE(), m.getPermeabilityM(), m.getElectricalConductivity(),
                            m.getMagneticConductivity()});
    }
    parallel_for(nx, [&](size_t i) {
      for (size_t q = i * ny * nz; q < (i + 1) * ny * nz; ++q) cell_mat[q] = vid[_voxel_index[q]];
    });
    std::fill(cell_disp.begin(), cell_disp.end(), -1);   // voxel materials are plain
  }

  // ---- coefficient table with per-cell overrides ------------------------
  std::vector<Tuple> table;
  for (const Props &p : mats) table.push_back(coefficients(p, dt, d));
  const size_t NX1 = nx + 1, NY1 = ny + 1, NZ1 = nz + 1;
  auto box_cell = [&](size_t i, size_t j, size_t k) { return (i * NY1 + j) * NZ1 + k; };
  auto base_mat = [&](size_t i, size_t j, size_t k) -> uint32_t {
    return (i < nx && j < ny && k < nz) ? cell_mat[(i * ny + j) * nz + k] : 0u;
  };
  std::unordered_map<size_t, Tuple> over;   // box cell -> modified tuple
  auto tuple_at = [&](size_t i, size_t j, size_t k) -> Tuple & {
    const size_t key = box_cell(i, j, k);
    auto it = over.find(key);
    if (it == over.end()) it = over.emplace(key, table[base_mat(i, j, k)]).first;
    return it->second;
  };

  // thin wires (ThinWire::correctFDTDCoff, thin_wire.cpp:39-129), in object order
  for (auto &o : _objects) {
    if (!o->isThinWire()) continue;
    const Cylinder &cy = dynamic_cast<const Cylinder &>(o->shape());
    auto g = gs.gridBox(cy);
    const size_t is = g[0], js = g[1], ks = g[2], ie = g[3], je = g[4], ke = g[5];
    const double r = cy.getRadius();
    const double dx = d[0], dy = d[1], dz = d[2];
    if (cy.getAxis() == Axis::X) {
      for (size_t i = is; i < ie; ++i) {
        Tuple &t = tuple_at(i, js, ks);
        t[0] = t[1] = t[2] = 0.0;
      }
      const double khy = dz * std::atan(dy / dy) / dy, khz = dy * std::atan(dz / dy) / dz;
      for (size_t i = is; i < ie; ++i)
        for (size_t k = ks - 1; k < ks + 1; ++k) {
          Tuple &t = tuple_at(i, js, k);
          t[14] = khy * 2 * t[14] / std::log(dz / r);   // chyex
        }
      for (size_t i = is; i < ie; ++i)
        for (size_t j = js - 1; j < js + 1; ++j) {
          Tuple &t = tuple_at(i, j, ks);
          t[16] = khz * 2 * t[16] / std::log(dy / r);   // chzex
        }
    } else if (cy.getAxis() == Axis::Y) {   // E coefficients untouched on this axis, as there
      const double khz = dx * std::atan(dz / dx) / dz, khx = dz * std::atan(dx / dz) / dx;
      for (size_t i = is - 1; i < is + 1; ++i)
        for (size_t j = js; j < je; ++j) {
          Tuple &t = tuple_at(i, j, ks);
          t[17] = khz * 2 * t[17] / std::log(dx / r);   // chzey
        }
      for (size_t j = js; j < je; ++j)
        for (size_t k = ks - 1; k < ks + 1; ++k) {
          Tuple &t = tuple_at(is, j, k);
          t[10] = khx * 2 * t[10] / std::log(dz / r);   // chxey
        }
    } else {
      for (size_t k = ks; k < ke; ++k) {
        Tuple &t = tuple_at(is, js, k);
        t[6] = t[7] = t[8] = 0.0;
      }
      const double khx = dy * std::atan(dx / dy) / dx, khy = dx * std::atan(dy / dx) / dy;
      for (size_t j = js - 1; j < js + 1; ++j)
        for (size_t k = ks; k < ke; ++k) {
          Tuple &t = tuple_at(is, j, k);
          t[11] = khx * 2 * t[11] / std::log(dy / r);   // chxez
        }
      for (size_t i = is - 1; i < is + 1; ++i)
        for (size_t k = ks; k < ke; ++k) {
          Tuple &t = tuple_at(i, js, k);
          t[13] = khy * 2 * t[13] / std::log(dx / r);   // chyez
        }
    }
  }

  // lumped elements
  std::vector<double> waveforms;
  int n_waveforms = 0;
  std::vector<xfdtd_injection> injections;
  std::vector<xfdtd_inductor_cell> inductors;
  for (auto &le : _lumped_elements) {
    auto g = gs.gridBox(le->cube());
    const size_t s[3] = {g[0], g[1], g[2]}, e[3] = {g[3], g[4], g[5]};
    const double n_i = static_cast<double>(e[0] - s[0]), n_j = static_cast<double>(e[1] - s[1]),
                 n_k = static_cast<double>(e[2] - s[2]);
    int comp;
    const CurrentSource *cs = dynamic_cast<const CurrentSource *>(le.get());
    const VoltageSource *vs = dynamic_cast<const VoltageSource *>(le.get());
    const Resistor *rs = dynamic_cast<const Resistor *>(le.get());
    const Capacitor *cp = dynamic_cast<const Capacitor *>(le.get());
    const Inductor *id = dynamic_cast<const Inductor *>(le.get());
    if (cs) comp = static_cast<int>(cs->getOrientation()) / 2;
    else if (vs) comp = static_cast<int>(vs->getOrientation()) / 2;
    else if (rs) comp = static_cast<int>(rs->getAxis());
    else if (cp) comp = static_cast<int>(cp->getAxis());
    else if (id) comp = static_cast<int>(id->getAxis());
    else throw std::runtime_error("unknown lumped element");
    const double along = comp == 0 ? n_i : (comp == 1 ? n_j : n_k);
    const double across = comp == 0 ? n_j * n_k : (comp == 1 ? n_i * n_k : n_i * n_j);
    if (along == 0 || across == 0) throw std::runtime_error("lumped element box is empty on the grid");
    // da, db: H-node sizes across, dc: E-node size along (uniform: the cell size)
    const double da = comp == 0 ? d[1] : (comp == 1 ? d[2] : d[0]);
    const double db = comp == 0 ? d[2] : (comp == 1 ? d[0] : d[1]);
    const double dc = d[comp];
    const int ce_i = 3 * comp, cha_i = 3 * comp + 1, chb_i = 3 * comp + 2;
    int wave_id = -1;
    double amp = 0, factor = 0;
    if (cs || vs) {
      const double R = cs ? cs->getResistance() : vs->getResistance();
      const Orientation ori = cs ? cs->getOrientation() : vs->getOrientation();
      factor = R * across / along;
      amp = (cs ? cs->waveform().getAmplitude() / across : vs->waveform().getAmplitude() / along);
      if (static_cast<int>(ori) % 2 == 0) amp *= -1;
      auto w = (cs ? cs->waveform() : vs->waveform()).clone();
      w->setAmplitude(amp);
      w->init(linspace(0.5 * dt, (static_cast<double>(_total) - 0.5) * dt, _total));
      wave_id = n_waveforms++;
      waveforms.insert(waveforms.end(), w->getValue().begin(), w->getValue().end());
    } else if (rs) {
      factor = rs->getResistance() * across / along;
    } else if (cp) {
      factor = cp->getCapacitance() * along / across;
    } else {
      factor = id->getInductance() * across / along;
    }
    for (size_t i = s[0]; i < e[0]; ++i)
      for (size_t j = s[1]; j < e[1]; ++j)
        for (size_t k = s[2]; k < e[2]; ++k) {
          const Props &pr = mats[base_mat(i, j, k)];
          const double ev = pr.eps, sv = pr.se;
          if (id) {   // inductor.cpp:66-100
            xfdtd_inductor_cell c{};
            c.comp = comp;
            c.i = static_cast<int64_t>(i);
            c.j = static_cast<int64_t>(j);
            c.k = static_cast<int64_t>(k);
            c.cjcec = dt * dc / (factor * da * db);
            c.cecjc = -(2 * dt) / (2 * ev + dt * sv);
            inductors.push_back(c);
            continue;
          }
          Tuple &t = tuple_at(i, j, k);
          if (cp) {   // capacitor.cpp:72, 100-120
            const double beta = 2 * factor * dc / (da * db);
            t[ce_i] = (2 * ev - dt * sv + beta) / (2 * ev + dt * sv + beta);
            t[cha_i] = -(2 * dt) / ((2 * ev + dt * sv + beta) * db);
            t[chb_i] = (2 * dt) / ((2 * ev + dt * sv + beta) * da);
            continue;
          }
          double beta, alpha = 0;
          if (vs) {   // voltage_source.cpp:126-128
            alpha = da * db * factor;
            beta = dt * dc / alpha;
          } else {    // current_source.cpp:112, resistor.cpp:66
            beta = (dt * dc) / (factor * da * db);
          }
          t[ce_i] = (2 * ev - dt * sv - beta) / (2 * ev + dt * sv + beta);
          t[cha_i] = -2 * dt / ((2 * ev + dt * sv + beta) * db);
          t[chb_i] = 2 * dt / ((2 * ev + dt * sv + beta) * da);
          if (cs || vs) {
            xfdtd_injection c{};
            c.comp = comp;
            c.waveform = wave_id;
            c.i = static_cast<int64_t>(i);
            c.j = static_cast<int64_t>(j);
            c.k = static_cast<int64_t>(k);
            c.coff = cs ? -2 * dt / ((2 * ev + dt * sv + beta) * (db * da))
                        : -2 * dt / ((2 * ev + dt * sv + beta) * alpha);
            injections.push_back(c);
          }
        }
  }

  // material index raster over the (nx+1)(ny+1)(nz+1) box, overrides interned
  std::map<Tuple, uint32_t> tuple_ids;
  for (uint32_t q = 0; q < table.size(); ++q) tuple_ids.emplace(table[q], q);
  std::vector<uint32_t> idx32(NX1 * NY1 * NZ1);
  parallel_for(NX1, [&](size_t i) {
    for (size_t j = 0; j < NY1; ++j)
      for (size_t k = 0; k < NZ1; ++k) idx32[box_cell(i, j, k)] = base_mat(i, j, k);
  });
  for (auto &kv : over) {
    auto it = tuple_ids.find(kv.second);
    uint32_t id;
    if (it == tuple_ids.end()) {
      id = static_cast<uint32_t>(table.size());
      table.push_back(kv.second);
      tuple_ids.emplace(kv.second, id);
    } else {
      id = it->second;
    }
    idx32[kv.first] = id;
  }
  const int index_bytes = table.size() <= 256 ? 1 : table.size() <= 65536 ? 2 : 4;
  std::vector<uint8_t> idx_bytes(idx32.size() * index_bytes);
  const size_t plane = NY1 * NZ1;
  if (index_bytes == 1)
    parallel_for(NX1, [&](size_t i) {
      for (size_t q = i * plane; q < (i + 1) * plane; ++q) idx_bytes[q] = static_cast<uint8_t>(idx32[q]);
    });
  else if (index_bytes == 2)
    parallel_for(NX1, [&](size_t i) {
      for (size_t q = i * plane; q < (i + 1) * plane; ++q) {
        const uint16_t v = static_cast<uint16_t>(idx32[q]);
        std::memcpy(idx_bytes.data() + 2 * q, &v, 2);
      }
    });
  else
    std::memcpy(idx_bytes.data(), idx32.data(), idx32.size() * 4);
  std::vector<double> coeff(table.size() * XFDTD_N_COEFF);
  for (size_t q = 0; q < table.size(); ++q)
    std::copy(table[q].begin(), table[q].end(), coeff.begin() + q * XFDTD_N_COEFF);

  xfdtd_plan_desc plan{};
  plan.nx = static_cast<int32_t>(nx);
  plan.ny = static_cast<int32_t>(ny);
  plan.nz = static_cast<int32_t>(nz);
  plan.precision = _precision == Precision::FP64 ? XFDTD_FP64 : XFDTD_FP32;
  plan.dt = dt;
  for (int a = 0; a < 3; ++a) plan.dl[a] = d[a];
  plan.total_steps = static_cast<int64_t>(_total);
  plan.flags = (_use_graph ? XFDTD_FLAG_GRAPH : 0) | (_profile ? XFDTD_FLAG_PROFILE : 0) |
               (_autotune ? XFDTD_FLAG_AUTOTUNE : 0) | (_fused == 0 ? XFDTD_FLAG_SPLIT_EH : 0) |
               (_fused == 1 ? XFDTD_FLAG_FUSED_EH : 0);
  plan.index_bytes = index_bytes;
  plan.device = _device;
  plan.n_materials = static_cast<int32_t>(table.size());
  plan.material_index = idx_bytes.data();
  plan.coeff_table = coeff.data();

  // ---- CPML -------------------------------------------------------------
  CpmlProfile prof[3];
  const size_t n_ax[3] = {nx, ny, nz};
  for (int a = 0; a < 3; ++a) {
    const PML *pn = nullptr, *pp = nullptr;
    for (auto &b : _boundaries) {
      const PML *p = dynamic_cast<const PML *>(b.get());
      if (!p) throw std::runtime_error("only PML boundaries are supported");
      const int o = static_cast<int>(p->getOrientation());
      if (o / 2 != a) continue;
      if (o % 2 == 0) {
        if (pn) throw std::runtime_error("two PML layers on the same face");
        pn = p;
      } else {
        if (pp) throw std::runtime_error("two PML layers on the same face");
        pp = p;
      }
    }
    CpmlProfile &cp = prof[a];
    const size_t n = n_ax[a];
    cp.slot_e.assign(n + 1, -1);
    cp.slot_h.assign(n + 1, -1);
    cp.b_e.assign(n + 1, 0.0); cp.a_e.assign(n + 1, 0.0); cp.rk_e.assign(n + 1, 1.0);
    cp.b_m.assign(n + 1, 0.0); cp.a_m.assign(n + 1, 0.0); cp.rk_m.assign(n + 1, 1.0);
    const int TN = pn ? pn->getSize() : 0, TP = pp ? pp->getSize() : 0;
    if (TN < 0 || TP < 0) throw std::runtime_error("negative PML thickness");
    if (static_cast<size_t>(TN + TP) >= n) throw std::runtime_error("PML layers overlap");
    std::vector<double> be, ae, ke, bm, am, km;
    if (pn) {   // N side: E at start+l+1, H at start+l, start = 0
      pmlLayers(*pn, d[a], dt, false, be, ae, ke, bm, am, km);
      for (int l = 0; l < TN; ++l) {
        const size_t ie = l + 1, ih = l;
        cp.slot_e[ie] = l; cp.b_e[ie] = be[l]; cp.a_e[ie] = ae[l]; cp.rk_e[ie] = 1.0 / ke[l];
        cp.slot_h[ih] = l; cp.b_m[ih] = bm[l]; cp.a_m[ih] = am[l]; cp.rk_m[ih] = 1.0 / km[l];
      }
    }
    if (pp) {   // P side: E and H at start+l, start = n - T
      pmlLayers(*pp, d[a], dt, true, be, ae, ke, bm, am, km);
      const size_t start = n - TP;
      for (int l = 0; l < TP; ++l) {
        const size_t q = start + l;
        cp.slot_e[q] = TN + l; cp.b_e[q] = be[l]; cp.a_e[q] = ae[l]; cp.rk_e[q] = 1.0 / ke[l];
        cp.slot_h[q] = TN + l; cp.b_m[q] = bm[l]; cp.a_m[q] = am[l]; cp.rk_m[q] = 1.0 / km[l];
      }
    }
    cp.layers = TN + TP;
    xfdtd_cpml_axis &ca = plan.cpml[a];
    ca.n_layers = cp.layers;
    ca.slot_e = cp.slot_e.data();
    ca.slot_h = cp.slot_h.data();
    ca.b_e = cp.b_e.data(); ca.a_e = cp.a_e.data(); ca.rk_e = cp.rk_e.data();
    ca.b_m = cp.b_m.data(); ca.a_m = cp.a_m.data(); ca.rk_m = cp.rk_m.data();
  }

  // ---- TFSF -------------------------------------------------------------
  std::vector<double> pf[3], ph[3], source;
  if (_tfsf) {
    TFSF &t = *_tfsf;
    auto [dx_, dy_, dz_] = t.getDistance();
    const size_t dist[3] = {dx_, dy_, dz_};
    size_t lo[3], hi[3], bn[3];
    for (int a = 0; a < 3; ++a) {
      if (2 * dist[a] >= n_ax[a]) throw std::runtime_error("TFSF box is empty");
      bn[a] = n_ax[a] - 2 * dist[a];
      lo[a] = dist[a];
      hi[a] = dist[a] + bn[a];
    }
    const double th = t.getIncidentTheta(), phi = t.getIncidentPhi(), psi = t.getIncidentPsi();
    const double st = std::sin(th), ct = std::cos(th), sp = std::sin(phi), cpv = std::cos(phi);
    const PointVector k = t.getKVector();
    // tfsf_3d.cpp:18-31
    const double u[3][3] = {{-sp, ct * cpv, st * cpv}, {cpv, ct * sp, st * sp}, {0, -st, ct}};
    const double ke[3] = {std::sin(psi), std::cos(psi), 0};
    double te[3], thv[3];
    for (int r = 0; r < 3; ++r) te[r] = u[r][0] * ke[0] + u[r][1] * ke[1] + u[r][2] * ke[2];
    thv[0] = k[1] * te[2] - k[2] * te[1];
    thv[1] = k[2] * te[0] - k[0] * te[2];
    thv[2] = k[0] * te[1] - k[1] * te[0];
    // tfsf_3d.cpp:47-57
    const double ratio_delta = 1 / std::sqrt(std::pow(std::sin(th), 4) * (std::pow(std::cos(phi), 4) + std::pow(std::sin(phi), 4)) +
                                             std::pow(std::cos(th), 4));
    // TFSF2D::init (tfsf_2d.cpp:44-46) takes sqrt(nz^2) where TFSF3D takes nz^2
    const double diagonal =
        two_d ? std::sqrt(std::pow(bn[0], 2) + std::pow(bn[1], 2) + std::sqrt(std::pow(bn[2], 2))) * ratio_delta
              : std::sqrt(std::pow(bn[0], 2) + std::pow(bn[1], 2) + std::pow(bn[2], 2)) * ratio_delta;
    const size_t L = static_cast<size_t>(std::ceil(diagonal)) + 4 + 1;
    // origin = box corner on the incoming side - 2 k / ratio_delta (:66-109;
    // 2-D: tfsf_2d.cpp:55-75, corner z = 0)
    double orig[3];
    for (int a = 0; a < 3; ++a)
      orig[a] = (k[a] >= 0 ? static_cast<double>(lo[a]) : static_cast<double>(hi[a])) - 2 * k[a] / ratio_delta;
    if (two_d) orig[2] = 0.0 - 2 * k[2] / ratio_delta;
    for (int a = 0; a < 3; ++a) {
      pf[a].resize(bn[a] + 1);
      ph[a].resize(bn[a] + 2);
      // the 2-D incident fields carry no z projection term (tfsf_2d.cpp:230-258):
      // zero tables add nothing to the 3-D projection sums
      const double kz = (two_d && a == 2) ? 0.0 : k[a];
      for (size_t i = 0; i < bn[a] + 1; ++i) pf[a][i] = ((i + lo[a]) - orig[a]) * kz * ratio_delta;
      for (size_t i = 0; i < bn[a] + 2; ++i) ph[a][i] = ((i + lo[a]) - orig[a] - 0.5) * kz * ratio_delta;
    }
    const double scaled_dl = d[0] / ratio_delta;
    // the incident wave: e0 * w(t dt), tfsf.cpp:51-52, 80-82
    std::vector<double> times(_total);
    for (size_t q = 0; q < _total; ++q) times[q] = static_cast<double>(q) * dt;
    t.waveform().init(times);
    source.resize(_total);
    for (size_t q = 0; q < _total; ++q) source[q] = t.getIncidentFieldAmplitude() * t.waveform()(q);
    xfdtd_tfsf_plan &tp = plan.tfsf;
    tp.enabled = two_d ? 2 : 1;
    tp.aux_len = static_cast<int32_t>(L);
    for (int a = 0; a < 3; ++a) {
      tp.lo[a] = static_cast<int64_t>(lo[a]);
      tp.hi[a] = static_cast<int64_t>(hi[a]);
      tp.proj_full[a] = pf[a].data();
      tp.proj_half[a] = ph[a].data();
      tp.transform_e[a] = te[a];
      tp.transform_h[a] = thv[a];
      tp.ca[a] = dt / (constant::EPSILON_0 * d[a]);
      tp.cb[a] = dt / (constant::MU_0 * d[a]);
    }
    tp.ceihi = -(dt / (constant::EPSILON_0 * scaled_dl));
    tp.chiei = -(dt / (constant::MU_0 * scaled_dl));
    tp.mur_c1 = (constant::C_0 * dt - scaled_dl) / (constant::C_0 * dt + scaled_dl);
    tp.mur_c2 = 2 * scaled_dl / (constant::C_0 * dt + scaled_dl);
    tp.source = source.data();
  }

  // ---- NF-FF ------------------------------------------------------------
  std::vector<double> phase_j, phase_m, wave_number;
  const NffftFd *nfd = dynamic_cast<const NffftFd *>(_nffft.get());
  const NffftBroadBand *nbb = dynamic_cast<const NffftBroadBand *>(_nffft.get());
  const double bb_dir[2] = {nbb ? nbb->getTheta() : 0.0, nbb ? nbb->getPhi() : 0.0};
  if (_nffft && !nfd && !nbb) throw std::runtime_error("unknown NFFFT type");
  if (nbb) {   // NffftBroadBand::init (nffft_broadband.cpp:31-95): every step's samples
    auto [dx_, dy_, dz_] = nbb->getDistance();
    const size_t dist[3] = {dx_, dy_, dz_};
    xfdtd_nffft_plan &np = plan.nffft;
    np.enabled = 2;
    for (int a = 0; a < 3; ++a) {
      if (2 * dist[a] >= n_ax[a]) throw std::runtime_error("NF-FF box is empty");
      np.lo[a] = static_cast<int64_t>(dist[a]);
      np.hi[a] = static_cast<int64_t>(n_ax[a] - dist[a]);
    }
    np.n_theta = np.n_phi = 1;
    np.theta = &bb_dir[0];
    np.phi = &bb_dir[1];
  }
  if (nfd) {
    auto [dx_, dy_, dz_] = nfd->getDistance();
    const size_t dist[3] = {dx_, dy_, dz_};
    xfdtd_nffft_plan &np = plan.nffft;
    np.enabled = 1;
    const auto &f = nfd->getFrequencies();
    np.n_freq = static_cast<int32_t>(f.size());
    for (int a = 0; a < 3; ++a) {
      if (2 * dist[a] >= n_ax[a]) throw std::runtime_error("NF-FF box is empty");
      np.lo[a] = static_cast<int64_t>(dist[a]);
      np.hi[a] = static_cast<int64_t>(n_ax[a] - dist[a]);
    }
    using namespace std::complex_literals;
    phase_j.resize(2 * f.size() * _total);
    phase_m.resize(2 * f.size() * _total);
    for (size_t n = 0; n < f.size(); ++n)
      for (size_t t = 0; t < _total; ++t) {   // nffft_fd.cpp:91-106
        const std::complex<double> pj = dt * std::exp(-1i * 2.0 * constant::PI * (f[n] * (t + 0.5) * dt));
        const std::complex<double> pm = dt * std::exp(-1i * 2.0 * constant::PI * (f[n] * t * dt));
        const size_t o = 2 * (n * _total + t);
        phase_j[o] = pj.real(); phase_j[o + 1] = pj.imag();
        phase_m[o] = pm.real(); phase_m[o + 1] = pm.imag();
      }
    wave_number.resize(f.size());
    for (size_t n = 0; n < f.size(); ++n) wave_number[n] = 2 * constant::PI * f[n] / constant::C_0;
    np.phase_j = phase_j.data();
    np.phase_m = phase_m.data();
    np.wave_number = wave_number.data();
    np.n_theta = static_cast<int32_t>(nfd->getTheta().size());
    np.n_phi = static_cast<int32_t>(nfd->getPhi().size());
    np.theta = nfd->getTheta().data();
    np.phi = nfd->getPhi().data();
  }

  // ---- monitors -> probe terms and snapshot series ----------------------
  std::vector<xfdtd_probe_term> terms;
  std::vector<xfdtd_snapshot_desc> series;
  _monitor_probe.clear();
  _monitor_series.clear();
  _monitor_box.clear();
  int probe = 0;
  const size_t comp_shape[6][3] = {{nx, ny + 1, nz + 1}, {nx + 1, ny, nz + 1}, {nx + 1, ny + 1, nz},
                                   {nx + 1, ny, nz},     {nx, ny + 1, nz},     {nx, ny, nz + 1}};
  // the component view of a field monitor (field_monitor.cpp:31-82,
  // 91-122): the grid box, 0 cells counting as 1, clipped to the array
  auto field_box = [&](const TimeDomainFieldMonitor &fm) {
    auto g = gs.gridBox(fm.cube());
    const size_t num[3] = {g[3] - g[0], g[4] - g[1], g[5] - g[2]};
    const int normal = fm.getPlaneType() == PlaneType::XY ? 2 : fm.getPlaneType() == PlaneType::YZ ? 0 : 1;
    if (num[normal] > 1) throw std::runtime_error("Error: invalid grid box");
    FieldBox b;
    b.comp = static_cast<int>(fm.getComponent());
    for (int a = 0; a < 3; ++a) {
      const size_t lim = comp_shape[b.comp][a];
      b.lo[a] = g[a];
      if (b.lo[a] >= lim) throw std::out_of_range("field monitor outside its component");
      b.n[a] = std::min(std::max<size_t>(num[a], 1), lim - b.lo[a]);
    }
    return b;
  };
  for (auto &m : _monitors) {
    _monitor_series.push_back(-1);
    _monitor_box.emplace_back();
    if (auto fm = dynamic_cast<const TimeDomainFieldMonitor *>(m.get())) {
      _monitor_box.back() = field_box(*fm);
      _monitor_probe.push_back(-1);
      continue;
    }
    if (auto mm = dynamic_cast<const MovieMonitor *>(m.get())) {   // movie_monitor.cpp:46-59
      auto fm = dynamic_cast<const TimeDomainFieldMonitor *>(&mm->getMonitor());
      if (!fm) throw std::runtime_error("a MovieMonitor runs on the GPU engine over a TimeDomainFieldMonitor only");
      if (mm->getPlotStep() == 0) throw std::invalid_argument("MovieMonitor plot step must be at least 1");
      const FieldBox b = field_box(*fm);
      xfdtd_snapshot_desc sd{};
      sd.comp = b.comp;
      for (int a = 0; a < 3; ++a) {
        sd.lo[a] = static_cast<int64_t>(b.lo[a]);
        sd.n[a] = static_cast<int64_t>(b.n[a]);
      }
      sd.every = static_cast<int64_t>(mm->getPlotStep());
      sd.last = static_cast<int64_t>(mm->getTotalTimeSteps()) - 1;
      _monitor_box.back() = b;
      _monitor_series.back() = static_cast<long>(series.size());
      _monitor_probe.push_back(-1);
      series.push_back(sd);
      continue;
    }
    auto g = gs.gridBox(m->cube());
    const size_t is = g[0], js = g[1], ks = g[2], ie = g[3], je = g[4], ke = g[5];
    auto term = [&](int comp, size_t i, size_t j, size_t k, double w) {
      xfdtd_probe_term t{};
      t.probe = probe;
      t.comp = comp;
      t.i = static_cast<int64_t>(i);
      t.j = static_cast<int64_t>(j);
      t.k = static_cast<int64_t>(k);
      t.weight = w;
      terms.push_back(t);
    };
    if (auto vm = dynamic_cast<const VoltageMonitor *>(m.get())) {   // voltage_monitor.cpp:25-97
      const int o = static_cast<int>(vm->getOrientation()), axis = o / 2;
      const double other = axis == 0 ? static_cast<double>((je - js) * (ke - ks))
                           : axis == 1 ? static_cast<double>((ie - is) * (ke - ks))
                                       : static_cast<double>((ie - is) * (je - js));
      double c = -d[axis] / other;
      if (o % 2 == 0) c *= -1;
      for (size_t i = is; i < ie; ++i)
        for (size_t j = js; j < je; ++j)
          for (size_t k = ks; k < ke; ++k) term(axis, i, j, k, c);
    } else if (auto cm = dynamic_cast<const CurrentMonitor *>(m.get())) {   // current_monitor.cpp:23-115
      const int o = static_cast<int>(cm->getOrientation()), axis = o / 2;
      const double pos = o % 2 == 0 ? -1 : 1;
      if (is == 0 || js == 0 || ks == 0) throw std::runtime_error("current monitor touches the grid edge");
      if (axis == 0) {
        for (size_t j = js; j <= je; ++j) { term(4, is, j, ks - 1, pos * d[1]); term(4, is, j, ke, -pos * d[1]); }
        for (size_t k = ks; k <= ke; ++k) { term(5, is, je, k, pos * d[2]); term(5, is, js - 1, k, -pos * d[2]); }
      } else if (axis == 1) {
        for (size_t k = ks; k <= ke; ++k) { term(5, is - 1, js, k, pos * d[2]); term(5, ie, js, k, -pos * d[2]); }
        for (size_t i = is; i <= ie; ++i) { term(3, i, js, ke, pos * d[0]); term(3, i, js, ks - 1, -pos * d[0]); }
      } else {
        for (size_t i = is; i <= ie; ++i) { term(3, i, js - 1, ks, pos * d[0]); term(3, i, je, ks, -pos * d[0]); }
        for (size_t j = js; j <= je; ++j) { term(4, ie, j, ks, pos * d[1]); term(4, is - 1, j, ks, -pos * d[1]); }
      }
    } else {
      throw std::runtime_error("unknown monitor type");
    }
    _monitor_probe.push_back(probe);
    ++probe;
  }
  _n_probes = static_cast<size_t>(probe);

  plan.n_waveforms = n_waveforms;
  plan.waveforms = waveforms.data();
  plan.n_injections = static_cast<int32_t>(injections.size());
  plan.injections = injections.data();
  plan.n_inductor_cells = static_cast<int32_t>(inductors.size());
  plan.inductor_cells = inductors.data();
  plan.n_probes = probe;
  plan.n_probe_terms = static_cast<int32_t>(terms.size());
  plan.probe_terms = terms.data();
  plan.n_snapshots = static_cast<int32_t>(series.size());
  plan.snapshots = series.data();

  // ---- dispersive media: the E components their recursions update --------
  // Simulation::updateEWithDispersiveMaterial (simulation_update.cpp:221-280):
  // each component over its main-update range, in the cells whose object is
  // a dispersive medium.  Outside the CPML only (the reference's PML would
  // add its psi terms with the cell's free-space coefficients), and with no
  // lumped element on them (its coefficients would override the medium's).
  std::vector<xfdtd_dispersive_cell> disp_cells;
  if (!cell_disp.empty()) {
    auto in_slab = [&](int a, size_t q) { return prof[a].layers && prof[a].slot_e[q] >= 0; };
    for (size_t i = 0; i < nx; ++i)
      for (size_t j = 0; j < ny; ++j)
        for (size_t k = 0; k < nz; ++k) {
          const int32_t m = cell_disp[(i * ny + j) * nz + k];
          if (m < 0) continue;
          if (in_slab(0, i) || in_slab(1, j) || in_slab(2, k))
            throw std::runtime_error("dispersive media must lie outside the CPML");
          const bool on[3] = {j >= 1 && k >= 1, i >= 1 && k >= 1, i >= 1 && j >= 1};
          for (int c = 0; c < 3; ++c)
            if (on[c])
              disp_cells.push_back(xfdtd_dispersive_cell{c, m, static_cast<int64_t>(i), static_cast<int64_t>(j),
                                                         static_cast<int64_t>(k)});
        }
    auto disp_at = [&](int64_t i, int64_t j, int64_t k) {
      return i >= 0 && j >= 0 && k >= 0 && static_cast<size_t>(i) < nx && static_cast<size_t>(j) < ny &&
             static_cast<size_t>(k) < nz && cell_disp[(i * ny + j) * nz + k] >= 0;
    };
    for (const auto &c : injections)
      if (disp_at(c.i, c.j, c.k)) throw std::runtime_error("a lumped element lies in a dispersive medium");
    for (const auto &c : inductors)
      if (disp_at(c.i, c.j, c.k)) throw std::runtime_error("a lumped element lies in a dispersive medium");
  }
  plan.n_disp_media = static_cast<int32_t>(disp_media.size());
  plan.disp_media = disp_media.data();
  plan.n_disp_cells = static_cast<int32_t>(disp_cells.size());
  plan.disp_cells = disp_cells.data();
  plan.disp_dl = d[0];

  xfdtd_handle *h = nullptr;
  const int rc = xfdtd_create(&plan, &h);
  if (rc != XFDTD_OK) {
    std::string msg = h ? xfdtd_last_error(h) : "no handle";
    if (h) xfdtd_destroy(h);
    throw std::runtime_error("GPU engine: " + msg + " (status " + std::to_string(rc) + ")");
  }
  _engine = h;
}

void Simulation::step(size_t n) {
  if (!_engine) throw std::runtime_error("Simulation::init has not been called");
  checkEngine(xfdtd_step(_engine, static_cast<int64_t>(n)), _engine);
}

size_t Simulation::getCurrentTimeStep() const {
  int64_t s = 0;
  if (_engine) xfdtd_current_step(_engine, &s);
  return static_cast<size_t>(s);
}

std::vector<double> Simulation::readField(int comp) const {
  if (!_engine) throw std::runtime_error("Simulation::init has not been called");
  const size_t s[6][3] = {{_nx, _ny + 1, _nz + 1}, {_nx + 1, _ny, _nz + 1}, {_nx + 1, _ny + 1, _nz},
                          {_nx + 1, _ny, _nz},     {_nx, _ny + 1, _nz},     {_nx, _ny, _nz + 1}};
  if (comp < 0 || comp > 5) throw std::invalid_argument("component must be 0..5");
  std::vector<double> v(s[comp][0] * s[comp][1] * s[comp][2]);
  checkEngine(xfdtd_read_field(_engine, comp, v.data(), static_cast<int64_t>(v.size())), _engine);
  return v;
}

std::vector<double> Simulation::monitorValues(size_t m) const {
  if (!_engine) throw std::runtime_error("Simulation::init has not been called");
  if (m >= _monitors.size() || _monitor_probe[m] < 0) throw std::invalid_argument("not a voltage or current monitor");
  std::vector<double> all(_n_probes * _total);
  checkEngine(xfdtd_read_probes(_engine, all.data(), static_cast<int64_t>(all.size())), _engine);
  const size_t p = static_cast<size_t>(_monitor_probe[m]);
  return std::vector<double>(all.begin() + p * _total, all.begin() + (p + 1) * _total);
}

std::array<size_t, 3> Simulation::fieldMonitorShape(size_t m) const {
  if (!_engine) throw std::runtime_error("Simulation::init has not been called");
  if (m >= _monitors.size() || _monitor_box[m].comp < 0) throw std::invalid_argument("not a field or movie monitor");
  const FieldBox &b = _monitor_box[m];
  return {b.n[0], b.n[1], b.n[2]};
}

std::array<size_t, 3> Simulation::fieldMonitorOrigin(size_t m) const {
  fieldMonitorShape(m);
  const FieldBox &b = _monitor_box[m];
  return {b.lo[0], b.lo[1], b.lo[2]};
}

std::vector<long long> Simulation::fieldMonitorSteps(size_t m) const {
  fieldMonitorShape(m);
  if (_monitor_series[m] < 0) return {-1};
  int64_t count = 0;
  const int s = static_cast<int>(_monitor_series[m]);
  checkEngine(xfdtd_snapshot_frames(_engine, s, &count, nullptr, 0), _engine);
  std::vector<int64_t> st(static_cast<size_t>(count));
  checkEngine(xfdtd_snapshot_frames(_engine, s, &count, st.data(), count), _engine);
  return std::vector<long long>(st.begin(), st.end());
}

std::vector<double> Simulation::fieldMonitorFrame(size_t m, size_t f) const {
  const auto shp = fieldMonitorShape(m);
  const FieldBox &b = _monitor_box[m];
  std::vector<double> out(shp[0] * shp[1] * shp[2]);
  if (_monitor_series[m] >= 0) {
    checkEngine(xfdtd_read_snapshot(_engine, static_cast<int>(_monitor_series[m]), static_cast<int64_t>(f), out.data(),
                                    static_cast<int64_t>(out.size())),
                _engine);
    return out;
  }
  if (f != 0) throw std::invalid_argument("a field monitor has one frame");
  const auto all = readField(b.comp);
  const size_t s1 = b.comp == 0 || b.comp == 2 || b.comp == 4 ? _ny + 1 : _ny;
  const size_t s2 = b.comp <= 1 || b.comp == 5 ? _nz + 1 : _nz;
  size_t q = 0;
  for (size_t i = 0; i < b.n[0]; ++i)
    for (size_t j = 0; j < b.n[1]; ++j)
      for (size_t k = 0; k < b.n[2]; ++k) out[q++] = all[((b.lo[0] + i) * s1 + b.lo[1] + j) * s2 + b.lo[2] + k];
  return out;
}

void Simulation::writeField(int comp, const std::vector<double> &values) {
  if (!_engine) throw std::runtime_error("Simulation::init has not been called");
  checkEngine(xfdtd_write_field(_engine, comp, values.data(), static_cast<int64_t>(values.size())), _engine);
}

std::vector<std::complex<double>> Simulation::farField(int which) const {
  const NffftFd *nfd = dynamic_cast<const NffftFd *>(_nffft.get());
  if (!_engine || !nfd) throw std::runtime_error("no NF-FF in this simulation");
  const size_t dirs = nfd->getFrequencies().size() * nfd->getTheta().size() * nfd->getPhi().size();
  std::vector<double> buf(2 * dirs);
  checkEngine(xfdtd_far_field(_engine, which, buf.data(), static_cast<int64_t>(buf.size())), _engine);
  std::vector<std::complex<double>> r(dirs);
  for (size_t q = 0; q < dirs; ++q) r[q] = {buf[2 * q], buf[2 * q + 1]};
  return r;
}

std::vector<double> Simulation::farFieldPower(int which) const {
  const NffftFd *nfd = dynamic_cast<const NffftFd *>(_nffft.get());
  if (!_engine || !nfd) throw std::runtime_error("no NF-FF in this simulation");
  const size_t dirs = nfd->getFrequencies().size() * nfd->getTheta().size() * nfd->getPhi().size();
  std::vector<double> buf(dirs);
  checkEngine(xfdtd_far_field(_engine, 8 + which, buf.data(), static_cast<int64_t>(buf.size())), _engine);
  return buf;
}

std::vector<std::complex<double>> Simulation::nffftAccumulator(int which) const {
  const NffftFd *nfd = dynamic_cast<const NffftFd *>(_nffft.get());
  if (!_engine || !nfd) throw std::runtime_error("no NF-FF in this simulation");
  auto [dx_, dy_, dz_] = nfd->getDistance();
  const size_t bx = _nx - 2 * dx_, by = _ny - 2 * dy_, bz = _nz - 2 * dz_;
  const size_t face[3] = {by * bz, bz * bx, bx * by};
  const size_t n = nfd->getFrequencies().size() * face[which / 8];
  std::vector<double> buf(2 * n);
  checkEngine(xfdtd_read_nffft(_engine, which, buf.data(), static_cast<int64_t>(buf.size())), _engine);
  std::vector<std::complex<double>> r(n);
  for (size_t q = 0; q < n; ++q) r[q] = {buf[2 * q], buf[2 * q + 1]};
  return r;
}

BroadbandFarField Simulation::broadbandFarField() const {
  const NffftBroadBand *nbb = dynamic_cast<const NffftBroadBand *>(_nffft.get());
  if (!_engine || !nbb) throw std::runtime_error("no broadband NF-FF in this simulation");
  const size_t N = 2 * _total - 1;
  std::vector<std::complex<double>> aux(6 * N);
  checkEngine(xfdtd_broadband_far_field(_engine, reinterpret_cast<double *>(aux.data()), static_cast<int64_t>(12 * N)),
              _engine);
  const std::complex<double> *n_x = &aux[0], *n_y = &aux[N], *n_z = &aux[2 * N], *l_x = &aux[3 * N],
                             *l_y = &aux[4 * N], *l_z = &aux[5 * N];
  BroadbandFarField r;
  // calculateFarField (nffft_broadband.cpp:343-371)
  const double fs = 1 / _dt;
  const double step = (fs / 2 - (-fs / 2)) / static_cast<double>(N - 1);
  r.frequencies.resize(N);
  r.wave_number.resize(N);
  for (size_t m = 0; m < N; ++m) {
    r.frequencies[m] = -fs / 2 + step * static_cast<double>(m);
    r.wave_number[m] = 2 * constant::PI * r.frequencies[m] / constant::C_0;
  }
  const double th = nbb->getTheta(), ph = nbb->getPhi();
  const double ct = std::cos(th), st = std::sin(th), cp = std::cos(ph), sp = std::sin(ph);
  using namespace std::complex_literals;
  for (auto *v : {&r.n_theta, &r.n_phi, &r.l_theta, &r.l_phi, &r.e_theta, &r.e_phi, &r.h_theta, &r.h_phi}) v->resize(N);
  r.power_theta.resize(N);
  r.power_phi.resize(N);
  const double eta = constant::ETA_0;
  for (size_t m = 0; m < N; ++m) {
    r.n_theta[m] = ct * cp * n_x[m] + ct * sp * n_y[m] - st * n_z[m];
    r.n_phi[m] = -sp * n_x[m] + cp * n_y[m];
    r.l_theta[m] = ct * cp * l_x[m] + ct * sp * l_y[m] - st * l_z[m];
    r.l_phi[m] = -sp * l_x[m] + cp * l_y[m];
    const double k = r.wave_number[m];
    r.e_theta[m] = (-1i * k) * (eta * r.n_theta[m] + r.l_phi[m]) / (4 * constant::PI);
    r.e_phi[m] = (1i * k) * (-eta * r.n_phi[m] + r.l_theta[m]) / (4 * constant::PI);
    r.h_theta[m] = (1i * k) * (r.n_phi[m] - r.l_theta[m] / eta) / (4 * constant::PI);
    r.h_phi[m] = (-1i * k) * (r.n_theta[m] + r.l_phi[m] / eta) / (4 * constant::PI);
    const double coff = std::pow(k, 2) / (32 * constant::PI * constant::PI * eta);
    r.power_theta[m] = coff * std::pow(std::abs(eta * r.n_theta[m] + r.l_phi[m]), 2);
    r.power_phi[m] = coff * std::pow(std::abs(-eta * r.n_phi[m] + r.l_theta[m]), 2);
  }
  return r;
}

std::vector<double> Simulation::rcsDb() const {
  const NffftFd *nfd = dynamic_cast<const NffftFd *>(_nffft.get());
  if (!nfd || !_tfsf) throw std::runtime_error("RCS needs a TFSF source and an NF-FF box");
  auto et = farField(0), ep = farField(1);
  auto inc = _tfsf->getIncidentWaveFourierTransform(nfd->getFrequencies());
  const size_t per_f = nfd->getTheta().size() * nfd->getPhi().size();
  std::vector<double> r(et.size());
  for (size_t q = 0; q < et.size(); ++q) {
    const double a = std::abs(inc[q / per_f]);
    r[q] = 10 * std::log10(4 * constant::PI * (std::norm(et[q]) + std::norm(ep[q])) / (a * a));
  }
  return r;
}

void Simulation::run(size_t total_time_steps) {
  init(total_time_steps);
  step(total_time_steps);
  outputData();
}

}  // namespace xfdtd

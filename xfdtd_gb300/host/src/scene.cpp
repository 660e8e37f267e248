// scene.cpp -- shapes, materials, objects, waveforms, sources and the uniform
// GridSpace of the reference's scene API.
#include <algorithm>
#include <cmath>

#include "xfdtd/xfdtd.h"

namespace xfdtd {

namespace {
// src/include/util/float_compare.h:9-24
bool isLessOrEqual(double a, double b, double eps = constant::TOLERABLE_EPSILON) {
  return (std::abs(a - b) < eps) ? true : (a < b);
}
bool isGreaterOrEqual(double a, double b, double eps = constant::TOLERABLE_EPSILON) {
  return (std::abs(a - b) < eps) ? true : (a > b);
}
}  // namespace

// src/shape/cube.cpp:27-37
bool Cube::isPointInside(const PointVector &p) const {
  return isLessOrEqual(_point[0], p[0]) && isLessOrEqual(_point[1], p[1]) && isLessOrEqual(_point[2], p[2]) &&
         isGreaterOrEqual(_point[0] + _size[0], p[0]) && isGreaterOrEqual(_point[1] + _size[1], p[1]) &&
         isGreaterOrEqual(_point[2] + _size[2], p[2]);
}

// src/shape/sphere.cpp:27-36
bool Sphere::isPointInside(const PointVector &p) const {
  const double dx = p[0] - _center[0], dy = p[1] - _center[1], dz = p[2] - _center[2];
  return isLessOrEqual(std::sqrt(dx * dx + dy * dy + dz * dz), _radius);
}
std::unique_ptr<Shape> Sphere::getWrappedBox() const {
  return std::make_unique<Cube>(PointVector{_center[0] - _radius, _center[1] - _radius, _center[2] - _radius},
                                PointVector{2 * _radius, 2 * _radius, 2 * _radius});
}

// src/shape/cylinder.cpp:26-66
bool Cylinder::isPointInside(const PointVector &p) const {
  if (!getWrappedBox()->isPointInside(p)) return false;
  const int a = static_cast<int>(_axis);
  const int a0 = a == 0 ? 1 : 0, a1 = a == 2 ? 1 : 2;
  const double dis = std::sqrt(std::pow(p[a0] - _center[a0], 2) + std::pow(p[a1] - _center[a1], 2));
  return isLessOrEqual(dis, _radius);
}
std::unique_ptr<Shape> Cylinder::getWrappedBox() const {
  PointVector pt, sz;
  for (int q = 0; q < 3; ++q) {
    if (q == static_cast<int>(_axis)) {
      pt[q] = _center[q] - _height / 2;
      sz[q] = _height;
    } else {
      pt[q] = _center[q] - _radius;
      sz[q] = 2 * _radius;
    }
  }
  return std::make_unique<Cube>(pt, sz);
}

// src/material/material.cpp:7-34
Material::Material(std::string_view name, float eps_r, float mu_r, double sigma_e, double sigma_m, bool is_dispersion)
    : _name{name}, _eps_r{eps_r}, _mu_r{mu_r}, _eps{_eps_r * constant::EPSILON_0}, _mu{_mu_r * constant::MU_0},
      _sigma_e{sigma_e}, _sigma_m{sigma_m}, _is_dispersion{is_dispersion} {}
Material Material::withExactPermittivity(std::string_view name, double eps_r, float mu_r, double sigma_e,
                                         double sigma_m) {
  Material m(name, static_cast<float>(eps_r), mu_r, sigma_e, sigma_m);
  m._eps = eps_r * constant::EPSILON_0;
  return m;
}
std::unique_ptr<Material> Material::createAir(const std::string &name) {
  return std::make_unique<Material>(name, 1, 1, 0, 0);
}
std::unique_ptr<Material> Material::createPEC() { return std::make_unique<Material>("XFDTD_PEC", 1, 1, 1e10, 0); }
std::unique_ptr<Material> Material::createPMC() { return std::make_unique<Material>("XFDTD_PMC", 1, 1, 1e10, 0); }

// src/object/object.cpp:12-47
Object::Object(std::string_view name, std::unique_ptr<Shape> shape, std::unique_ptr<Material> material)
    : _name{name}, _shape{std::move(shape)}, _material{std::move(material)} {}
Object::Object(std::string_view name, std::unique_ptr<Shape> shape, Material material)
    : _name{name}, _shape{std::move(shape)}, _material{std::make_unique<Material>(std::move(material))} {}
Object::Object(const Object &o)
    : _name{o._name}, _shape{o._shape->clone()}, _material{std::make_unique<Material>(*o._material)} {}
Object &Object::operator=(const Object &o) {
  if (this != &o) {
    _name = o._name;
    _shape = o._shape->clone();
    _material = std::make_unique<Material>(*o._material);
  }
  return *this;
}

// src/object/thin_wire.cpp:10-15 (the material is a placeholder there too)
ThinWire::ThinWire(const std::string &name, std::unique_ptr<Cylinder> shape)
    : Object(name, std::move(shape), Material::createAir("placeholder_wire")) {}

// ---------------------------------------------------------------- waveforms
void Waveform::init(const std::vector<double> &t) {  // custom_waveform.cpp:13-20 shape
  std::vector<double> v(t.size());
  for (size_t i = 0; i < t.size(); ++i) v[i] = getValueByTime(t[i]);
  setValue(std::move(v));
}
std::vector<std::complex<double>> Waveform::getFourierTransform(const std::vector<double> &freqs, double dt) const {
  // util/dft.h:11-27
  using namespace std::complex_literals;
  std::vector<std::complex<double>> r(freqs.size());
  for (size_t i = 0; i < freqs.size(); ++i) {
    std::complex<double> sum{0.0, 0.0};
    for (size_t j = 0; j < _value.size(); ++j) {
      const double t = j * dt;
      sum += _value[j] * std::exp(-2.0 * 1i * constant::PI * freqs[i] * t);
    }
    r[i] = sum * dt;
  }
  return r;
}
double GaussianWaveform::getValueByTime(double t) const {  // gaussian_waveform.cpp:18-24
  return getAmplitude() * std::exp(-std::pow((t - _t_0) / _tau, 2));
}
void GaussianWaveform::init(const std::vector<double> &t) {
  std::vector<double> v(t.size());
  for (size_t i = 0; i < t.size(); ++i) v[i] = getAmplitude() * std::exp(-std::pow((t[i] - _t_0) / _tau, 2));
  setValue(std::move(v));
}
double CosineModulatedGaussianWaveform::getValueByTime(double t) const {
  return getAmplitude() * std::cos(2 * constant::PI * _f * (t - _t_0)) * std::exp(-std::pow((t - _t_0) / _tau, 2));
}
void CosineModulatedGaussianWaveform::init(const std::vector<double> &t) {
  std::vector<double> v(t.size());
  for (size_t i = 0; i < t.size(); ++i)
    v[i] = getAmplitude() * std::cos(2 * constant::PI * _f * (t[i] - _t_0)) *
           std::exp(-std::pow((t[i] - _t_0) / _tau, 2));
  setValue(std::move(v));
}
double SinusoidalWaveform::getValueByTime(double t) const {
  return getAmplitude() * std::sin(2 * constant::PI * _frequency * t + _phase);
}
void SinusoidalWaveform::init(const std::vector<double> &t) {
  std::vector<double> v(t.size());
  for (size_t i = 0; i < t.size(); ++i) v[i] = getAmplitude() * std::sin(2 * constant::PI * _frequency * t[i] + _phase);
  setValue(std::move(v));
}

// ---------------------------------------------------------------- TFSF base
// src/tfsf/tfsf.cpp:15-33
TFSF::TFSF(SpatialIndex dx, SpatialIndex dy, SpatialIndex dz, double e_0, double theta_inc, double phi_inc, double psi,
           std::shared_ptr<Waveform> waveform)
    : _distance_x{dx}, _distance_y{dy}, _distance_z{dz}, _e_0{e_0}, _theta_inc{theta_inc}, _phi_inc{phi_inc},
      _psi{psi}, _waveform{std::move(waveform)} {
  _k = {std::sin(theta_inc) * std::cos(phi_inc), std::sin(theta_inc) * std::sin(phi_inc), std::cos(theta_inc)};
}
std::vector<std::complex<double>> TFSF::getIncidentWaveFourierTransform(const std::vector<double> &freqs) const {
  auto r = _waveform->getFourierTransform(freqs, _dt);
  for (auto &v : r) v *= _e_0;
  return r;
}

// ----------------------------------------------------------- lumped sources
// src/lumped_element/current_source.cpp:5-16, voltage_source.cpp:15-26
CurrentSource::CurrentSource(std::unique_ptr<Cube> cube, Orientation orientation, double resistance,
                             std::unique_ptr<Waveform> waveform)
    : LumpedElement{std::move(cube)}, _orientation{orientation}, _resistance{resistance},
      _waveform{std::move(waveform)} {
  if (_resistance == 0) _resistance = 1e-20;  // avoid a division by zero, as there
}
CurrentSource::CurrentSource(const CurrentSource &o)
    : LumpedElement{o}, _orientation{o._orientation}, _resistance{o._resistance}, _waveform{o._waveform->clone()} {}
VoltageSource::VoltageSource(std::unique_ptr<Cube> cube, Orientation orientation, double resistance,
                             std::unique_ptr<Waveform> waveform)
    : LumpedElement{std::move(cube)}, _orientation{orientation}, _resistance{resistance},
      _waveform{std::move(waveform)} {
  if (_resistance == 0) _resistance = 1e-20;
}
VoltageSource::VoltageSource(const VoltageSource &o)
    : LumpedElement{o}, _orientation{o._orientation}, _resistance{o._resistance}, _waveform{o._waveform->clone()} {}

// ------------------------------------------------------------------ GridSpace
GridSpace::GridSpace(double dl) {
  for (int a = 0; a < 3; ++a) {
    _base[a] = dl;
    _mn[a] = std::numeric_limits<double>::max();
    _mx[a] = std::numeric_limits<double>::min();   // as grid_space.cpp:24-26
  }
}

void GridSpace::resize(const double *mn, const double *mx) {  // resizeSpaceSize, grid_space.cpp:576-618
  for (int a = 0; a < 3; ++a) {
    if (_mn[a] > mn[a]) _mn[a] = mn[a];
    if (_mx[a] < mx[a]) _mx[a] = mx[a];
  }
  for (int a = 0; a < 3; ++a) {
    size_t n = static_cast<size_t>(std::round((_mx[a] - _mn[a]) / _base[a]));
    if (_mx[a] < _mn[a]) n = 1;
    _n[a] = std::max(_n[a], n);
  }
}

void GridSpace::calculateSpaceSize(const Cube &b) {
  if (_ready) throw std::runtime_error("GridSpace is ready");
  const double mn[3] = {b.getXmin(), b.getYmin(), b.getZmin()};
  const double mx[3] = {b.getXmax(), b.getYmax(), b.getZmax()};
  resize(mn, mx);
}

void GridSpace::extendBoundary(Orientation o, double size) {  // extendBoundary{XN..ZP}, :364-464
  if (_ready) throw std::runtime_error("GridSpace is ready");
  const int axis = static_cast<int>(o) / 2;
  if (_n[axis] <= 1) throw std::runtime_error("GridSpace is not extended");
  if (size < 0) throw std::runtime_error("size is less than 0");
  double mn[3] = {_mn[0], _mn[1], _mn[2]}, mx[3] = {_mx[0], _mx[1], _mx[2]};
  if (static_cast<int>(o) % 2 == 0) mn[axis] = _mn[axis] - size;
  else mx[axis] = _mx[axis] + size;
  resize(mn, mx);
}

void GridSpace::generateUniformGridSpace() {  // :501-538, :625-638, :737-757
  if (_ready) throw std::runtime_error("GridSpace is ready");
  for (int a = 0; a < 3; ++a) _n[a] = std::max<size_t>(_n[a], 1);
  // :513-533: three extended axes make the 3-D grid; the 2-D grid of the
  // TMz path has x and y extended and nz = 1 (the 1-D grid is not built)
  if (_n[0] > 1 && _n[1] > 1 && _n[2] > 1) _dim = 3;
  else if (_n[0] > 1 && _n[1] > 1 && _n[2] == 1) _dim = 2;
  else throw std::runtime_error("the GPU engine runs the 3-D grid and the 2-D (nz = 1) grid only");
  for (int a = 0; a < 3; ++a) {
    _ec[a].resize(_n[a] + 1);
    for (size_t i = 0; i <= _n[a]; ++i) _ec[a][i] = _mn[a] + static_cast<double>(i) * _base[a];
    _hc[a].resize(_n[a]);
    for (size_t i = 0; i < _n[a]; ++i) _hc[a][i] = (_ec[a][i] + _ec[a][i + 1]) / 2;
  }
  _ready = true;
}

size_t GridSpace::nearest(int a, double x) const {  // argmin |e_node - x|, first minimum
  if (x < _mn[a]) throw std::out_of_range("coordinate is out of range");
  size_t best = 0;
  double bd = std::abs(_ec[a][0] - x);
  for (size_t i = 1; i < _ec[a].size(); ++i) {
    const double d = std::abs(_ec[a][i] - x);
    if (d < bd) {
      bd = d;
      best = i;
    }
  }
  return best;
}

std::array<size_t, 6> GridSpace::gridBox(const Shape &shape) const {
  auto w = shape.getWrappedBox();
  const Cube *c = dynamic_cast<const Cube *>(w.get());
  if (!c) throw std::runtime_error("Shape Type Error");
  const double mn[3] = {c->getXmin(), c->getYmin(), c->getZmin()};
  const double mx[3] = {c->getXmax(), c->getYmax(), c->getZmax()};
  std::array<size_t, 6> r{};
  for (int a = 0; a < 3; ++a) {
    r[a] = nearest(a, mn[a]);
    r[3 + a] = nearest(a, mx[a]);
    if (r[3 + a] < r[a]) throw std::range_error("end < start");
  }
  return r;
}

void checkEngine(int status, xfdtd_handle *h);

}  // namespace xfdtd

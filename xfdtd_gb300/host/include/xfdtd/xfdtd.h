// xfdtd.h -- the reference XFDTD C++ scene API (Mrwatermolen/XFDTD), kept
// class for class so that a program written against the reference builds
// against this library, plus the GB300 engine underneath it.
//
// Kept: class names, constructor signatures, argument order and defaults of
//   Simulation       src/include/simulation/simulation.h:27-66
//   Object, ThinWire src/include/object/object.h:17-20, thin_wire.h
//   Shape, Cube, Sphere, Cylinder   src/include/shape/*.h
//   Material         src/include/material/material.h:14-78
//   Boundary, PML    src/include/boundary/{boundary.h,perfect_match_layer.h}
//   Waveform family  src/include/waveform/*.h
//   TFSF, TFSF3D     src/include/tfsf/{tfsf.h,tfsf_3d.h}
//   NFFFT, NffftFd   src/include/nffft/{nffft.h,nffft_fd.h}
//   LumpedElement, CurrentSource, VoltageSource, Resistor, Capacitor,
//   Inductor         src/include/lumped_element/*.h
//   Monitor, VoltageMonitor, CurrentMonitor   src/include/monitor/*.h
// and the .npy outputs of NffftFd::outputData / Monitor::outputData.
//
// Changed: xtensor types in signatures become std::vector<double> /
// std::array; PointVector is std::array<double, 3>.  The per-step virtual
// hooks (Boundary::updateE/H, TFSF::updateE/H, NFFFT::update, Monitor::update,
// LumpedElement::correctE/H) are not called per step: Simulation lowers the
// whole scene to one plan and the GPU engine runs the loop.  A user subclass
// that overrides those hooks is therefore not supported.
#pragma once

#include <array>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <iostream>   // the reference's headers bring it in, and its drivers print with std::cout
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <string_view>
#include <tuple>
#include <vector>

struct xfdtd_handle;

namespace xfdtd {

// src/include/util/constant.h:10-29
namespace constant {
inline constexpr double PI{3.14159265358979323846};
inline constexpr double EPSILON_0{8.854187817e-12};
inline constexpr double MU_0{4 * PI * 1e-7};
inline constexpr double SQUARED_C_0{1 / (EPSILON_0 * MU_0)};
inline const double ETA_0{std::sqrt(MU_0 / EPSILON_0)};
inline const double C_0{std::sqrt(SQUARED_C_0)};
inline constexpr double TOLERABLE_EPSILON{10 * std::numeric_limits<double>::epsilon()};
}  // namespace constant

using PointVector = std::array<double, 3>;
using SpatialIndex = size_t;

// The angle lists the reference's drivers build with xt::linspace(start,
// stop, num, endpoint) (examples/3d_pec_sphere_bistatic_rcs.cpp:78), as a
// std::vector: element i is start + i * step, step = (stop - start) /
// (num - 1) with the end point and (stop - start) / num without it.
inline std::vector<double> linspace(double start, double stop, size_t num, bool endpoint = true) {
  std::vector<double> v(num);
  const size_t div = endpoint ? (num > 1 ? num - 1 : 1) : num;
  const double step = num ? (stop - start) / static_cast<double>(div) : 0.0;
  for (size_t i = 0; i < num; ++i) v[i] = start + static_cast<double>(i) * step;
  return v;
}
enum class Orientation { XN, XP, YN, YP, ZN, ZP };
enum class Axis { X, Y, Z };
// src/include/electromagnetic_field/electromagnetic_field.h:8,
// src/include/util/type_define.h:30
enum class EMComponent { EX, EY, EZ, HX, HY, HZ };
enum class PlaneType { XY, YZ, ZX };

// GB300 engine precision (extension).
enum class Precision { FP64, FP32 };

// ----------------------------------------------------------------- shapes
class Cube;
class Shape {
 public:
  virtual ~Shape() = default;
  virtual bool isPointInside(const PointVector &point) const = 0;
  virtual std::unique_ptr<Shape> getWrappedBox() const = 0;
  virtual std::unique_ptr<Shape> clone() const = 0;
};

class Cube : public Shape {
 public:
  Cube(PointVector point, PointVector size) : _point{point}, _size{size} {}
  bool isPointInside(const PointVector &point) const override;
  std::unique_ptr<Shape> getWrappedBox() const override { return std::make_unique<Cube>(_point, _size); }
  std::unique_ptr<Shape> clone() const override { return std::make_unique<Cube>(*this); }
  double getXmin() const { return _point[0]; }
  double getXmax() const { return _point[0] + _size[0]; }
  double getYmin() const { return _point[1]; }
  double getYmax() const { return _point[1] + _size[1]; }
  double getZmin() const { return _point[2]; }
  double getZmax() const { return _point[2] + _size[2]; }
  PointVector getSize() const { return _size; }
  PointVector getPoint() const { return _point; }

 private:
  PointVector _point, _size;
};

class Sphere : public Shape {
 public:
  Sphere(PointVector center, double radius) : _center{center}, _radius{radius} {}
  bool isPointInside(const PointVector &point) const override;
  std::unique_ptr<Shape> getWrappedBox() const override;
  std::unique_ptr<Shape> clone() const override { return std::make_unique<Sphere>(*this); }
  double getRadius() const { return _radius; }
  PointVector getCenter() const { return _center; }

 private:
  PointVector _center;
  double _radius;
};

class Cylinder : public Shape {
 public:
  Cylinder(Axis axis, PointVector center, double radius, double height)
      : _axis{axis}, _center{center}, _radius{radius}, _height{height} {}
  bool isPointInside(const PointVector &point) const override;
  std::unique_ptr<Shape> getWrappedBox() const override;
  std::unique_ptr<Shape> clone() const override { return std::make_unique<Cylinder>(*this); }
  Axis getAxis() const { return _axis; }
  double getRadius() const { return _radius; }
  double getHeight() const { return _height; }
  PointVector getCenter() const { return _center; }

 private:
  Axis _axis;
  PointVector _center;
  double _radius, _height;
};

// --------------------------------------------------------------- material
class Material {
 public:
  Material(std::string_view name, float eps_r, float mu_r, double sigma_e, double sigma_m,
           bool is_dispersion = false);
  // A material whose relative permittivity is kept in double (the
  // constructor above takes eps_r as float, as the reference's does): for
  // finite-difference gradient checks.  No counterpart in the reference.
  static Material withExactPermittivity(std::string_view name, double eps_r, float mu_r, double sigma_e,
                                        double sigma_m);
  static std::unique_ptr<Material> createAir(const std::string &name = "XFDTD_AIR");
  static std::unique_ptr<Material> createPEC();
  static std::unique_ptr<Material> createPMC();
  double getPermittivityE() const { return _eps; }
  double getPermeabilityM() const { return _mu; }
  double getElectricalConductivity() const { return _sigma_e; }
  double getMagneticConductivity() const { return _sigma_m; }
  std::tuple<double, double, double, double> getElectromagneticProperties() const {
    return {_eps, _mu, _sigma_e, _sigma_m};
  }
  bool isDispersion() const { return _is_dispersion; }
  float getEpsR() const { return _eps_r; }
  float getMuR() const { return _mu_r; }
  const std::string &getName() const { return _name; }
  // A linear dispersive medium's kind (0 none, 1 Lorentz, 2 Drude, 3 Debye)
  // and parameters, kept in the base so that an Object's copy keeps them.
  int dispersionKind() const { return _disp_kind; }
  const std::array<double, 4> &dispersionParams() const { return _disp_p; }

 protected:
  void setDispersion(int kind, std::array<double, 4> p) {
    _disp_kind = kind;
    _disp_p = p;
  }

 private:
  std::string _name;
  float _eps_r, _mu_r;
  double _eps, _mu, _sigma_e, _sigma_m;
  bool _is_dispersion;
  int _disp_kind = 0;
  std::array<double, 4> _disp_p{0, 0, 0, 0};
};

// Linear dispersive media (src/include/material/dispersive_material.h):
// eps_r = mu_r = 1, the frequency dependence in an E recursion per medium
// (src/material/dispersive_material.cpp).  Uniform grids with dx = dy = dz
// only, and outside the CPML.  The reference throws on them at
// Object::init (object.cpp:109-110); the GPU engine runs them.
class LinearDispersiveMaterial : public Material {
 public:
  explicit LinearDispersiveMaterial(std::string_view name, float eps_r = 1, float mu_r = 1, double sigma_e = 0,
                                    double sigma_m = 0)
      : Material(name, eps_r, mu_r, sigma_e, sigma_m, true) {}
};
class LorentzMedium : public LinearDispersiveMaterial {
 public:
  LorentzMedium(std::string_view name, double eps_s, double eps_inf, double omega_p, double nv, double sigma_e = 0,
                double sigma_m = 0)
      : LinearDispersiveMaterial(name, 1, 1, sigma_e, sigma_m) {
    setDispersion(1, {eps_s, eps_inf, omega_p, nv});
  }
};
class DrudeMedium : public LinearDispersiveMaterial {
 public:
  DrudeMedium(std::string_view name, double eps_inf, double pole_omega, double nv, double sigma_e = 0,
              double sigma_m = 0)
      : LinearDispersiveMaterial(name, 1, 1, sigma_e, sigma_m) {
    setDispersion(2, {eps_inf, pole_omega, nv, 0});
  }
};
class DebyMedium : public LinearDispersiveMaterial {
 public:
  DebyMedium(std::string_view name, double eps_s, double eps_inf, double tau, double sigma_e = 0,
             double sigma_m = 0)
      : LinearDispersiveMaterial(name, 1, 1, sigma_e, sigma_m) {
    setDispersion(3, {eps_s, eps_inf, tau, 0});
  }
};

// ----------------------------------------------------------------- object
class Object {
 public:
  Object(std::string_view name, std::unique_ptr<Shape> shape, std::unique_ptr<Material> material);
  Object(std::string_view name, std::unique_ptr<Shape> shape, Material material);
  Object(const Object &other);
  Object &operator=(const Object &other);
  Object(Object &&) noexcept = default;
  Object &operator=(Object &&) noexcept = default;
  virtual ~Object() = default;
  std::unique_ptr<Shape> getWrappedBox() const { return _shape->getWrappedBox(); }
  std::unique_ptr<Shape> getShape() const { return _shape->clone(); }
  const Shape &shape() const { return *_shape; }
  const Material &material() const { return *_material; }
  bool isDispersion() const { return _material->isDispersion(); }
  virtual bool isThinWire() const { return false; }
  const std::string &getName() const { return _name; }

 private:
  std::string _name;
  std::unique_ptr<Shape> _shape;
  std::unique_ptr<Material> _material;
};

class ThinWire : public Object {
 public:
  ThinWire(const std::string &name, std::unique_ptr<Cylinder> shape);
  bool isThinWire() const override { return true; }
};

// --------------------------------------------------------------- boundary
class Boundary {
 public:
  virtual ~Boundary() = default;
  virtual Orientation getOrientation() const = 0;
  virtual int getSize() const = 0;
};

class PML : public Boundary {
 public:
  PML(Orientation orientation, int thickness, int order = 4, double sigma_ratio = 1, double alpha_min = 0,
      double alpha_max = 0.05, double kappa_max = 10)
      : _orientation{orientation}, _thickness{thickness}, _order{order}, _sigma_ratio{sigma_ratio},
        _alpha_min{alpha_min}, _alpha_max{alpha_max}, _kappa_max{kappa_max} {}
  Orientation getOrientation() const override { return _orientation; }
  int getSize() const override { return _thickness; }
  int getOrder() const { return _order; }
  double getSigmaRatio() const { return _sigma_ratio; }
  double getAlphaMin() const { return _alpha_min; }
  double getAlphaMax() const { return _alpha_max; }
  double getKappaMax() const { return _kappa_max; }

 private:
  Orientation _orientation;
  int _thickness, _order;
  double _sigma_ratio, _alpha_min, _alpha_max, _kappa_max;
};

// --------------------------------------------------------------- waveform
class Waveform {
 public:
  explicit Waveform(double amplitude) : _amplitude{amplitude} {}
  Waveform() = default;
  virtual ~Waveform() = default;
  virtual std::unique_ptr<Waveform> clone() const = 0;
  // Samples amplitude * f(t) at the given times (Waveform::init).
  virtual void init(const std::vector<double> &time_array);
  virtual double getValueByTime(double time) const = 0;
  const std::vector<double> &getValue() const { return _value; }
  double operator()(size_t i) const { return _value.at(i); }
  double getAmplitude() const { return _amplitude; }
  void setAmplitude(double a) { _amplitude = a; }
  std::vector<std::complex<double>> getFourierTransform(const std::vector<double> &frequencies, double dt) const;

 protected:
  void setValue(std::vector<double> v) { _value = std::move(v); }

 private:
  double _amplitude{1.0};
  std::vector<double> _value;
};

class GaussianWaveform : public Waveform {
 public:
  GaussianWaveform(double amplitude, double tau, double t_0) : Waveform{amplitude}, _tau{tau}, _t_0{t_0} {}
  GaussianWaveform(double tau, double t_0) : _tau{tau}, _t_0{t_0} {}
  std::unique_ptr<Waveform> clone() const override { return std::make_unique<GaussianWaveform>(*this); }
  double getValueByTime(double t) const override;
  void init(const std::vector<double> &time_array) override;

 private:
  double _tau, _t_0;
};

class CosineModulatedGaussianWaveform : public Waveform {
 public:
  CosineModulatedGaussianWaveform(double amplitude, double tau, double t_0, double modulation_frequency)
      : Waveform{amplitude}, _tau{tau}, _t_0{t_0}, _f{modulation_frequency} {}
  CosineModulatedGaussianWaveform(double tau, double t_0, double modulation_frequency)
      : _tau{tau}, _t_0{t_0}, _f{modulation_frequency} {}
  std::unique_ptr<Waveform> clone() const override {
    return std::make_unique<CosineModulatedGaussianWaveform>(*this);
  }
  double getValueByTime(double t) const override;
  void init(const std::vector<double> &time_array) override;

 private:
  double _tau, _t_0, _f;
};

class SinusoidalWaveform : public Waveform {
 public:
  SinusoidalWaveform(double amplitude, double frequency, double phase)
      : Waveform(amplitude), _frequency(frequency), _phase(phase) {}
  SinusoidalWaveform(double frequency, double phase) : _frequency(frequency), _phase(phase) {}
  std::unique_ptr<Waveform> clone() const override { return std::make_unique<SinusoidalWaveform>(*this); }
  double getValueByTime(double t) const override;
  void init(const std::vector<double> &time_array) override;

 private:
  double _frequency, _phase;
};

class CustomWaveform : public Waveform {
 public:
  CustomWaveform(double amplitude, std::function<double(double)> f) : Waveform(amplitude), _f(std::move(f)) {}
  std::unique_ptr<Waveform> clone() const override { return std::make_unique<CustomWaveform>(*this); }
  double getValueByTime(double t) const override { return getAmplitude() * _f(t); }

 private:
  std::function<double(double)> _f;
};

// ------------------------------------------------------------------- TFSF
class TFSF {
 public:
  TFSF(SpatialIndex distance_x, SpatialIndex distance_y, SpatialIndex distance_z, double e_0, double theta_inc,
       double phi_inc, double psi, std::shared_ptr<Waveform> waveform);
  virtual ~TFSF() = default;
  std::tuple<SpatialIndex, SpatialIndex, SpatialIndex> getDistance() const {
    return {_distance_x, _distance_y, _distance_z};
  }
  double getIncidentFieldAmplitude() const { return _e_0; }
  double getIncidentTheta() const { return _theta_inc; }
  double getIncidentPhi() const { return _phi_inc; }
  double getIncidentPsi() const { return _psi; }
  PointVector getKVector() const { return _k; }
  Waveform &waveform() const { return *_waveform; }
  // dt * sum_t e0 w[t] exp(-i 2 pi f t dt) over the sampled incident wave
  // (TFSF::getIncidentWaveFourierTransform, tfsf.cpp:63-66; valid after run/init).
  std::vector<std::complex<double>> getIncidentWaveFourierTransform(const std::vector<double> &frequencies) const;
  void bindTimeStep(double dt) { _dt = dt; }

 private:
  SpatialIndex _distance_x, _distance_y, _distance_z;
  double _e_0, _theta_inc, _phi_inc, _psi;
  PointVector _k;
  std::shared_ptr<Waveform> _waveform;
  double _dt{0};
};

class TFSF3D : public TFSF {
 public:
  TFSF3D(SpatialIndex distance_x, SpatialIndex distance_y, SpatialIndex distance_z, double e_0, double theta_inc,
         double phi_inc, double psi, std::shared_ptr<Waveform> waveform)
      : TFSF(distance_x, distance_y, distance_z, e_0, theta_inc, phi_inc, psi, std::move(waveform)) {}
};

// The plane wave of the 2-D (nz = 1) TMz grid (src/include/tfsf/tfsf_2d.h:8-10,
// src/tfsf/tfsf_2d.cpp:7-10): the TFSF base with theta = pi / 2, psi = 0
// and no z offset; Ez, Hx and Hy corrections on the x and y faces only.
class TFSF2D : public TFSF {
 public:
  TFSF2D(SpatialIndex distance_x, SpatialIndex distance_y, double phi_inc, double ez_i0,
         std::shared_ptr<Waveform> waveform)
      : TFSF(distance_x, distance_y, 0, ez_i0, constant::PI / 2, phi_inc, 0, std::move(waveform)) {}
};

// ------------------------------------------------------------------ NF-FF
class NFFFT {
 public:
  NFFFT(SpatialIndex distance_x, SpatialIndex distance_y, SpatialIndex distance_z, std::string output_dir_path)
      : _distance_x{distance_x}, _distance_y{distance_y}, _distance_z{distance_z},
        _output_dir_path{std::move(output_dir_path)} {}
  virtual ~NFFFT() = default;
  std::tuple<SpatialIndex, SpatialIndex, SpatialIndex> getDistance() const {
    return {_distance_x, _distance_y, _distance_z};
  }
  const std::string &getOutputDirPath() const { return _output_dir_path; }
  void setOutputDirPath(const std::string &d) { _output_dir_path = d; }

 private:
  SpatialIndex _distance_x, _distance_y, _distance_z;
  std::string _output_dir_path;
};

class NffftFd : public NFFFT {
 public:
  NffftFd(SpatialIndex distance_x, SpatialIndex distance_y, SpatialIndex distance_z, std::vector<double> frequencies,
          std::vector<double> theta, std::vector<double> phi, std::string output_dir_path)
      : NFFFT(distance_x, distance_y, distance_z, std::move(output_dir_path)), _frequencies{std::move(frequencies)},
        _theta{std::move(theta)}, _phi{std::move(phi)} {}
  NffftFd(SpatialIndex distance_x, SpatialIndex distance_y, SpatialIndex distance_z, double frequency,
          std::vector<double> theta, std::vector<double> phi, std::string output_dir_path)
      : NffftFd(distance_x, distance_y, distance_z, std::vector<double>{frequency}, std::move(theta), std::move(phi),
                std::move(output_dir_path)) {}
  const std::vector<double> &getFrequencies() const { return _frequencies; }
  const std::vector<double> &getTheta() const { return _theta; }
  const std::vector<double> &getPhi() const { return _phi; }

 private:
  std::vector<double> _frequencies, _theta, _phi;
};

// NffftBroadBand (src/include/nffft/nffft_broadband.h,
// src/nffft/nffft_broadband.cpp): the far field in one direction (theta,
// phi) over the whole band of the run: every step's surface samples are
// kept, and at the end each is Fourier transformed over N = 2T-1 points
// (zero-padded), phase-shifted by its path delay and summed.  The outputs
// are arrays over the N fftshifted bins, labelled by linspace(-fs/2, fs/2,
// N) with fs = 1/dt, as calculateFarField labels them.
class NffftBroadBand : public NFFFT {
 public:
  NffftBroadBand(SpatialIndex distance_x, SpatialIndex distance_y, SpatialIndex distance_z, double theta, double phi,
                 std::string output_dir_path)
      : NFFFT(distance_x, distance_y, distance_z, std::move(output_dir_path)), _theta{theta}, _phi{phi} {}
  double getTheta() const { return _theta; }
  double getPhi() const { return _phi; }

 private:
  double _theta, _phi;
};

// The far field of a broadband NF-FF over its N bins
// (NffftBroadBand::calculateFarField, nffft_broadband.cpp:343-371).
struct BroadbandFarField {
  std::vector<double> frequencies, wave_number;
  std::vector<std::complex<double>> n_theta, n_phi, l_theta, l_phi;
  std::vector<std::complex<double>> e_theta, e_phi, h_theta, h_phi;
  std::vector<double> power_theta, power_phi;
};

// ---------------------------------------------------------- lumped element
class LumpedElement {
 public:
  explicit LumpedElement(std::unique_ptr<Cube> cube) : _cube{std::move(cube)} {}
  LumpedElement(const LumpedElement &o) : _cube{std::make_unique<Cube>(*o._cube)} {}
  virtual ~LumpedElement() = default;
  const Cube &cube() const { return *_cube; }

 private:
  std::unique_ptr<Cube> _cube;
};

class CurrentSource : public LumpedElement {
 public:
  CurrentSource(std::unique_ptr<Cube> cube, Orientation orientation, double resistance,
                std::unique_ptr<Waveform> waveform);
  CurrentSource(const CurrentSource &o);
  Orientation getOrientation() const { return _orientation; }
  double getResistance() const { return _resistance; }
  Waveform &waveform() const { return *_waveform; }

 private:
  Orientation _orientation;
  double _resistance;
  std::unique_ptr<Waveform> _waveform;
};

class VoltageSource : public LumpedElement {
 public:
  VoltageSource(std::unique_ptr<Cube> cube, Orientation orientation, double resistance,
                std::unique_ptr<Waveform> waveform);
  VoltageSource(const VoltageSource &o);
  Orientation getOrientation() const { return _orientation; }
  double getResistance() const { return _resistance; }
  Waveform &waveform() const { return *_waveform; }

 private:
  Orientation _orientation;
  double _resistance;
  std::unique_ptr<Waveform> _waveform;
};

class Resistor : public LumpedElement {
 public:
  Resistor(std::unique_ptr<Cube> cube, Axis axis, double resistance)
      : LumpedElement{std::move(cube)}, _axis{axis}, _resistance{resistance} {}
  Axis getAxis() const { return _axis; }
  double getResistance() const { return _resistance; }

 private:
  Axis _axis;
  double _resistance;
};

class Capacitor : public LumpedElement {
 public:
  Capacitor(std::unique_ptr<Cube> cube, Axis axis, double capacitance)
      : LumpedElement{std::move(cube)}, _axis{axis}, _capacitance{capacitance} {}
  Axis getAxis() const { return _axis; }
  double getCapacitance() const { return _capacitance; }

 private:
  Axis _axis;
  double _capacitance;
};

class Inductor : public LumpedElement {
 public:
  Inductor(std::unique_ptr<Cube> cube, Axis axis, double inductance)
      : LumpedElement{std::move(cube)}, _axis{axis}, _inductance{inductance} {}
  Axis getAxis() const { return _axis; }
  double getInductance() const { return _inductance; }

 private:
  Axis _axis;
  double _inductance;
};

// ----------------------------------------------------------------- monitor
class Monitor {
 public:
  Monitor(std::unique_ptr<Cube> cube, std::string output_dir_path, std::string output_file_name)
      : _cube{std::move(cube)}, _dir{std::move(output_dir_path)}, _file{std::move(output_file_name)} {}
  Monitor(const Monitor &o) : _cube{std::make_unique<Cube>(*o._cube)}, _dir{o._dir}, _file{o._file} {}
  virtual ~Monitor() = default;
  const Cube &cube() const { return *_cube; }
  const std::string &getOutputPath() const { return _dir; }
  const std::string &getOutputFileName() const { return _file; }
  void setOutputDirPath(const std::string &d) { _dir = d; }
  void setOutputFileName(const std::string &f) { _file = f; }
  // Time series recorded by the last run (one value per step).
  const std::vector<double> &getValue() const { return _value; }
  double getValue(size_t i) const { return _value.at(i); }
  void setValue(std::vector<double> v) { _value = std::move(v); }

 private:
  std::unique_ptr<Cube> _cube;
  std::string _dir, _file;
  std::vector<double> _value;
};

class VoltageMonitor : public Monitor {
 public:
  VoltageMonitor(std::unique_ptr<Cube> shape, Orientation orientation, std::string output_dir_path,
                 std::string output_file_name)
      : Monitor{std::move(shape), std::move(output_dir_path), std::move(output_file_name)},
        _orientation{orientation} {}
  Orientation getOrientation() const { return _orientation; }

 private:
  Orientation _orientation;
};

class CurrentMonitor : public Monitor {
 public:
  CurrentMonitor(std::unique_ptr<Cube> shape, Orientation orientation, std::string output_dir_path,
                 std::string output_file_name)
      : Monitor{std::move(shape), std::move(output_dir_path), std::move(output_file_name)},
        _orientation{orientation} {}
  Orientation getOrientation() const { return _orientation; }

 private:
  Orientation _orientation;
};

// TimeDomainFieldMonitor (src/include/monitor/field_monitor.h,
// src/monitor/field_monitor.cpp): component `component` over the cube's
// grid box (an extent of 0 cells counts as 1), written by outputData as a
// 3-D .npy of the field after the last step.  The plane type is checked as
// the reference checks it (field_monitor.cpp:31-82): a monitor thicker than
// one cell across its plane is an error.
class TimeDomainFieldMonitor : public Monitor {
 public:
  TimeDomainFieldMonitor(std::unique_ptr<Cube> shape, PlaneType plane_type, EMComponent component,
                         std::string output_dir_path, std::string output_file_name)
      : Monitor{std::move(shape), std::move(output_dir_path), std::move(output_file_name)},
        _plane_type{plane_type},
        _component{component} {}
  PlaneType getPlaneType() const { return _plane_type; }
  EMComponent getComponent() const { return _component; }

 private:
  PlaneType _plane_type;
  EMComponent _component;
};

// MovieMonitor (src/include/monitor/movie_monitor.h,
// src/monitor/movie_monitor.cpp:46-59) over a TimeDomainFieldMonitor: a
// frame of the field after every step t with t % plot_step == 0 and after
// step total_time_steps - 1, written by outputData as <dir>/NNNN.npy (the
// step, four digits zero-padded) in the field monitor's directory.  The
// reference writes each frame during the run; here the frames stay in
// device memory until outputData.  Other monitors cannot be wrapped.
class MovieMonitor : public Monitor {
 public:
  MovieMonitor(std::unique_ptr<Monitor> monitor, size_t total_time_steps, size_t plot_step = 30)
      : Monitor{std::make_unique<Cube>(monitor->cube()), monitor->getOutputPath(), monitor->getOutputFileName()},
        _monitor{std::move(monitor)},
        _total_time_steps{total_time_steps},
        _plot_step{plot_step} {}
  const Monitor &getMonitor() const { return *_monitor; }
  size_t getTotalTimeSteps() const { return _total_time_steps; }
  size_t getPlotStep() const { return _plot_step; }
  void setPlotStep(size_t plot_step) { _plot_step = plot_step; }

 private:
  std::shared_ptr<Monitor> _monitor;
  size_t _total_time_steps;
  size_t _plot_step;
};

// ----------------------------------------------------------------- network
// dt * sum_j x[j] exp(-i 2 pi f j dt) for each f (src/include/util/dft.h:11-27).
std::vector<std::complex<double>> dft(const std::vector<double> &x, double dt, const std::vector<double> &frequencies);

// Port (src/include/network/port.h, src/network/port.cpp): the incident and
// reflected waves a = (V + Z I) / (2 sqrt(Re Z)), b = (V - conj(Z) I) /
// (2 sqrt(Re Z)) from the DFTs of its monitors' series.
class Port {
 public:
  Port(int index, std::complex<double> impedance, bool is_activated_source, std::shared_ptr<VoltageMonitor> voltage,
       std::shared_ptr<CurrentMonitor> current)
      : _index{index},
        _impedance{impedance},
        _is_activated_source{is_activated_source},
        _voltage{std::move(voltage)},
        _current{std::move(current)} {}
  void calculateSParameter(const std::vector<double> &frequencies, double dt);
  int getPortIndex() const { return _index; }
  bool isActivatedSource() const { return _is_activated_source; }
  std::complex<double> getImpedance() const { return _impedance; }
  const std::shared_ptr<VoltageMonitor> &getVoltageMonitor() const { return _voltage; }
  const std::shared_ptr<CurrentMonitor> &getCurrentMonitor() const { return _current; }
  const std::vector<std::complex<double>> &getA() const { return _a; }
  const std::vector<std::complex<double>> &getB() const { return _b; }

 private:
  int _index;
  std::complex<double> _impedance;
  bool _is_activated_source;
  std::shared_ptr<VoltageMonitor> _voltage;
  std::shared_ptr<CurrentMonitor> _current;
  std::vector<std::complex<double>> _a, _b;
};

// Network (src/include/network/network.h, src/network/network.cpp): for
// every activated port i and every port j, S[10 j + i] = b_j / a_i, by the
// ports' indices; outputData writes each as s<key>.npy, the frequencies
// stacked over the values (a complex (2, n_freq) array).
class Network {
 public:
  Network(std::vector<std::unique_ptr<Port>> ports, std::vector<double> frequencies, std::string output_path)
      : _ports{std::move(ports)}, _frequencies{std::move(frequencies)}, _output_path{std::move(output_path)} {}
  // Computes the S-parameters from the ports' monitor series (which
  // Simulation::outputData fills).
  void calculate(double dt);
  const std::vector<std::unique_ptr<Port>> &getPorts() const { return _ports; }
  const std::vector<double> &getFrequencies() const { return _frequencies; }
  const std::string &getOutputPath() const { return _output_path; }
  void setOutputPath(const std::string &p) { _output_path = p; }
  const std::map<int, std::vector<std::complex<double>>> &getSParameters() const { return _s_parameters; }

 private:
  std::vector<std::unique_ptr<Port>> _ports;
  std::vector<double> _frequencies;
  std::string _output_path;
  std::map<int, std::vector<std::complex<double>>> _s_parameters;
};

// -------------------------------------------------------------- grid space
// Uniform GridSpace (src/grid/grid_space.cpp:14-757, uniform path only).
class GridSpace {
 public:
  explicit GridSpace(double dl);
  void calculateSpaceSize(const Cube &box);
  void extendBoundary(Orientation o, double size);
  void generateUniformGridSpace();
  size_t n(int axis) const { return _n[axis]; }
  // 3 or 2 (GridSpace::Dimension, grid_space.cpp:513-533): the 2-D grid
  // has x and y extended and nz = 1
  int dim() const { return _dim; }
  double base(int axis) const { return _base[axis]; }
  double eNode(int axis, size_t i) const { return _ec[axis][i]; }
  double hNode(int axis, size_t i) const { return _hc[axis][i]; }
  const std::vector<double> &eNodes(int axis) const { return _ec[axis]; }
  const std::vector<double> &hNodes(int axis) const { return _hc[axis]; }
  // nearest E node (handleTransform*, grid_space.cpp:551-574)
  size_t nearest(int axis, double x) const;
  // [start, end) index box of a shape's wrapped cube (getGridBox, :306-329)
  std::array<size_t, 6> gridBox(const Shape &shape) const;

 private:
  double _base[3];
  double _mn[3], _mx[3];
  size_t _n[3] = {0, 0, 0};
  int _dim = 0;
  bool _ready = false;
  std::vector<double> _ec[3], _hc[3];
  void resize(const double *mn, const double *mx);
};

// --------------------------------------------------------------- simulation
class Simulation {
 public:
  inline static constexpr float DEFAULT_CFL{0.99};

  explicit Simulation(double cell_size, float cfl = DEFAULT_CFL);
  Simulation(double cell_size, std::vector<std::shared_ptr<Object>> objects,
             std::vector<std::shared_ptr<Boundary>> boundaries, std::unique_ptr<TFSF> tfsf, float cfl = DEFAULT_CFL);
  Simulation(double cell_size, std::vector<std::shared_ptr<Object>> objects,
             std::vector<std::shared_ptr<Boundary>> boundaries, std::unique_ptr<TFSF> tfsf,
             std::unique_ptr<NFFFT> nffft, float cfl = DEFAULT_CFL);
  Simulation(double cell_size, std::vector<std::shared_ptr<Object>> objects,
             std::vector<std::shared_ptr<LumpedElement>> lumped_elements,
             std::vector<std::shared_ptr<Boundary>> boundaries = {}, std::vector<std::shared_ptr<Monitor>> monitor = {},
             float cfl = DEFAULT_CFL);
  Simulation(double cell_size, std::vector<std::shared_ptr<Object>> objects,
             std::vector<std::shared_ptr<Monitor>> monitors = {}, float cfl = DEFAULT_CFL);
  // simulation.h:46-49 (the network's ports use monitors of the list)
  Simulation(double cell_size, std::vector<std::shared_ptr<Object>> objects,
             std::vector<std::shared_ptr<LumpedElement>> lumped_elements,
             std::vector<std::shared_ptr<Boundary>> boundaries, std::vector<std::shared_ptr<Monitor>> monitors,
             std::unique_ptr<Network> network, float cfl = DEFAULT_CFL);
  ~Simulation();
  Simulation(const Simulation &) = delete;
  Simulation &operator=(const Simulation &) = delete;

  void addObject(std::shared_ptr<Object> object);
  void addBoundary(std::shared_ptr<Boundary> boundary);
  void addLumpedElement(std::shared_ptr<LumpedElement> lumped_element);
  void addTFSFSource(std::shared_ptr<TFSF> tfsf);
  void addNFFFT(std::shared_ptr<NFFFT> nffft);
  void addMonitor(std::shared_ptr<Monitor> monitor);
  NFFFT *getNFFFT() const { return _nffft.get(); }
  void addNetwork(std::shared_ptr<Network> network) { _network = std::move(network); }
  Network *getNetwork() const { return _network.get(); }
  // The network's S-parameters from the monitor series recorded so far.
  const std::map<int, std::vector<std::complex<double>>> &sParameters();

  // Simulation::run (simulation_update.cpp:5-40): init, the loop, outputData.
  void run(size_t total_time_steps);
  // Builds the grid and the plan only and writes the counts
  // (Simulation::checkRun, simulation.cpp:98-113).
  void checkRun(size_t total_time_steps);

  // ---- GB300 extensions -------------------------------------------------
  void setPrecision(Precision p) { _precision = p; }
  Precision getPrecision() const { return _precision; }
  void setUseGraph(bool g) { _use_graph = g; }
  void setProfile(bool p) { _profile = p; }
  void setDevice(int d) { _device = d; }
  // Time the volume-kernel variants at init and keep the fastest (default on).
  void setAutotune(bool a) { _autotune = a; }
  // Volume kernels: 1 = always the fused E/H sweep, 0 = always separate
  // in-place E and H kernels, -1 (default) = the autotuner picks the faster.
  // Plans with lumped elements always run the split kernels.
  void setFusedSweep(int mode) { _fused = mode; }
  // One material per cell, applied after all objects (see xfdtd_scene.h).
  void setVoxelMaterials(std::vector<Material> materials, std::vector<uint16_t> index, std::array<size_t, 3> shape);
  void setVoxelMaterials(std::vector<Material> materials, std::vector<uint32_t> index, std::array<size_t, 3> shape);
  // Split run(): init once, step in pieces, read state, output at the end.
  void init(size_t total_time_steps);
  void step(size_t n);
  void outputData();
  size_t getCurrentTimeStep() const;
  size_t getTotalTimeSteps() const { return _total; }
  // Field component c (0 Ex .. 5 Hz) in the reference's component shape.
  std::vector<double> readField(int comp) const;
  void writeField(int comp, const std::vector<double> &values);
  // Far-field array `which` (0 e_theta .. 7 l_phi complex, 8/9 power).
  std::vector<std::complex<double>> farField(int which) const;
  std::vector<double> farFieldPower(int which) const;
  std::vector<std::complex<double>> nffftAccumulator(int which) const;
  // Time series of monitor m (a voltage or current monitor), one value per
  // step.
  std::vector<double> monitorValues(size_t m) const;
  // A field or movie monitor m: its box shape, and the steps of its frames
  // (a field monitor has one frame, the current field, step -1).
  std::array<size_t, 3> fieldMonitorShape(size_t m) const;
  std::array<size_t, 3> fieldMonitorOrigin(size_t m) const;
  std::vector<long long> fieldMonitorSteps(size_t m) const;
  // Frame f of field or movie monitor m, [n0][n1][n2].
  std::vector<double> fieldMonitorFrame(size_t m, size_t f) const;
  // The broadband NF-FF's far field from the steps run so far.
  BroadbandFarField broadbandFarField() const;
  // Bistatic RCS in dB over (frequency, theta, phi):
  // 10 log10(4 pi (|E_theta|^2 + |E_phi|^2) / |E_inc(f)|^2).
  std::vector<double> rcsDb() const;
  xfdtd_handle *engine() const { return _engine; }

  double getDt() const { return _dt; }
  SpatialIndex getNx() const { return _nx; }
  SpatialIndex getNy() const { return _ny; }
  SpatialIndex getNz() const { return _nz; }

 private:
  double _cell_size;
  float _cfl;
  std::vector<std::shared_ptr<Object>> _objects;
  std::vector<std::shared_ptr<Boundary>> _boundaries;
  std::vector<std::shared_ptr<LumpedElement>> _lumped_elements;
  std::vector<std::shared_ptr<Monitor>> _monitors;
  std::shared_ptr<TFSF> _tfsf;
  std::shared_ptr<NFFFT> _nffft;
  std::shared_ptr<Network> _network;
  std::vector<Material> _voxel_materials;
  std::vector<uint32_t> _voxel_index;
  std::array<size_t, 3> _voxel_shape{0, 0, 0};

  Precision _precision{Precision::FP64};
  bool _use_graph{true};
  bool _profile{false};
  int _device{0};
  int _fused{-1};
  bool _autotune{true};
  size_t _total{0};
  size_t _nx{0}, _ny{0}, _nz{0};
  double _dt{0};
  xfdtd_handle *_engine{nullptr};
  // per monitor: its probe index (voltage, current) or -1; its snapshot
  // series (movie) or -1; the component and box of a field monitor
  struct FieldBox {
    int comp = -1;
    size_t lo[3] = {0, 0, 0}, n[3] = {0, 0, 0};
  };
  std::vector<long> _monitor_probe, _monitor_series;
  std::vector<FieldBox> _monitor_box;
  size_t _n_probes{0};
  void release();
};

// Throws std::runtime_error with the engine's message on a non-zero status.
void checkEngine(int status, xfdtd_handle *h);

}  // namespace xfdtd

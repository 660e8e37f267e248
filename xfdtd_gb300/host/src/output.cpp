// output.cpp -- .npy outputs of the reference (NffftFd::outputData,
// src/nffft/nffft_fd.cpp:579-634; VoltageMonitor / CurrentMonitor ::outputData,
// src/monitor/voltage_monitor.cpp:99-120, current_monitor.cpp:117-140;
// TimeDomainFieldMonitor::outputData, src/monitor/field_monitor.cpp:91-122;
// MovieMonitor::update, src/monitor/movie_monitor.cpp:46-59;
// Network::outputData, src/network/network.cpp:27-60;
// NffftBroadBand::outputData, src/nffft/nffft_broadband.cpp:156-200) and
// Simulation::checkRun (src/simulation/simulation.cpp:98-113).
#include <cstdio>
#include <filesystem>
#include <iomanip>
#include <fstream>
#include <iostream>
#include <sstream>

#include "../../../include/xfdtd_cuda.h"
#include "xfdtd/xfdtd.h"

namespace xfdtd {

namespace {

// Minimal .npy (format 1.0) writer: little-endian '<f8' or '<c16', C order.
void writeNpy(const std::filesystem::path &path, const void *data, size_t elem_bytes, const char *descr,
              const std::vector<size_t> &shape) {
  std::ostringstream hdr;
  hdr << "{'descr': '" << descr << "', 'fortran_order': False, 'shape': (";
  for (size_t q = 0; q < shape.size(); ++q) hdr << shape[q] << (shape.size() == 1 || q + 1 < shape.size() ? ", " : "");
  hdr << "), }";
  std::string h = hdr.str();
  const size_t total = 10 + h.size() + 1;
  const size_t pad = (64 - total % 64) % 64;
  h.append(pad, ' ');
  h.push_back('\n');
  std::ofstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot write " + path.string());
  const char magic[] = {'\x93', 'N', 'U', 'M', 'P', 'Y', 1, 0};
  f.write(magic, 8);
  const uint16_t len = static_cast<uint16_t>(h.size());
  const unsigned char l2[2] = {static_cast<unsigned char>(len & 0xff), static_cast<unsigned char>(len >> 8)};
  f.write(reinterpret_cast<const char *>(l2), 2);
  f.write(h.data(), static_cast<std::streamsize>(h.size()));
  size_t n = 1;
  for (size_t s : shape) n *= s;
  f.write(static_cast<const char *>(data), static_cast<std::streamsize>(n * elem_bytes));
}

bool ensureDir(const std::filesystem::path &p) {
  if (p.empty()) return true;
  if (std::filesystem::exists(p)) return true;
  try {
    std::filesystem::create_directories(p);
  } catch (const std::exception &) {
    std::cerr << "Error: cannot create directory " << p.string() << '\n';
    return false;
  }
  return true;
}


}  // namespace

void Simulation::outputData() {
  if (!_engine) throw std::runtime_error("Simulation::init has not been called");
  // voltage and current monitors: stack(time, value) -> (2, N)
  if (_n_probes) {
    std::vector<double> all(_n_probes * _total);
    checkEngine(xfdtd_read_probes(_engine, all.data(), static_cast<int64_t>(all.size())), _engine);
    for (size_t m = 0; m < _monitors.size(); ++m) {
      if (_monitor_probe[m] < 0) continue;
      const size_t p = static_cast<size_t>(_monitor_probe[m]);
      std::vector<double> v(all.begin() + p * _total, all.begin() + (p + 1) * _total);
      _monitors[m]->setValue(v);
      const std::string &dir = _monitors[m]->getOutputPath();
      if (dir.empty()) continue;
      const bool current = dynamic_cast<const CurrentMonitor *>(_monitors[m].get()) != nullptr;
      auto t = current ? linspace(0.5 * _dt, (_total + 0.5) * _dt, _total) : linspace(0.0, _total * _dt, _total);
      if (!ensureDir(dir)) continue;
      std::vector<double> st(2 * _total);
      std::copy(t.begin(), t.end(), st.begin());
      std::copy(v.begin(), v.end(), st.begin() + _total);
      writeNpy(std::filesystem::path(dir) / _monitors[m]->getOutputFileName(), st.data(), 8, "<f8", {2, _total});
    }
  }
  // field monitors: the component over the box after the last step; movie
  // monitors: one NNNN.npy per recorded frame
  for (size_t m = 0; m < _monitors.size(); ++m) {
    if (_monitor_box[m].comp < 0) continue;
    const std::string &dir = _monitors[m]->getOutputPath();
    if (dir.empty() || !ensureDir(dir)) continue;
    const auto shp = fieldMonitorShape(m);
    const std::vector<size_t> shape{shp[0], shp[1], shp[2]};
    if (_monitor_series[m] < 0) {
      const auto v = fieldMonitorFrame(m, 0);
      writeNpy(std::filesystem::path(dir) / _monitors[m]->getOutputFileName(), v.data(), 8, "<f8", shape);
      continue;
    }
    const auto steps = fieldMonitorSteps(m);
    const long long done = static_cast<long long>(getCurrentTimeStep());
    for (size_t f = 0; f < steps.size(); ++f) {
      if (steps[f] >= done) continue;   // not run yet
      std::ostringstream name;
      name << std::setw(4) << std::setfill('0') << steps[f] << ".npy";
      const auto v = fieldMonitorFrame(m, f);
      writeNpy(std::filesystem::path(dir) / name.str(), v.data(), 8, "<f8", shape);
    }
  }
  // network: s<key>.npy = stack(frequencies, S) as complex (2, n_freq)
  if (_network && !_network->getOutputPath().empty() && ensureDir(_network->getOutputPath())) {
    const auto &sp = sParameters();
    const auto &fr = _network->getFrequencies();
    for (const auto &e : sp) {
      std::vector<std::complex<double>> st(2 * fr.size());
      for (size_t q = 0; q < fr.size(); ++q) {
        st[q] = {fr[q], 0.0};
        st[fr.size() + q] = e.second[q];
      }
      writeNpy(std::filesystem::path(_network->getOutputPath()) / ("s" + std::to_string(e.first) + ".npy"), st.data(),
               16, "<c16", {2, fr.size()});
    }
  }
  const NffftBroadBand *nbb = dynamic_cast<const NffftBroadBand *>(_nffft.get());
  if (nbb && !nbb->getOutputDirPath().empty() && ensureDir(nbb->getOutputDirPath())) {
    const std::filesystem::path out{nbb->getOutputDirPath()};
    const auto ff = broadbandFarField();
    const size_t N = ff.frequencies.size();
    {   // outputFarFieldParameters (:466-476)
      std::ofstream w{out / "far_field_parameter.dat"};
      w << "Fs:\t" << 1 / _dt << '\n';
      w << "number of samples:\t" << N << '\n';
      w << "Theta:\n" << nbb->getTheta() << '\n';
      w << "Phi:\n" << nbb->getPhi() << '\n';
    }
    writeNpy(out / "e_theta.npy", ff.e_theta.data(), 16, "<c16", {N});
    writeNpy(out / "e_phi.npy", ff.e_phi.data(), 16, "<c16", {N});
    writeNpy(out / "h_theta.npy", ff.h_theta.data(), 16, "<c16", {N});
    writeNpy(out / "h_phi.npy", ff.h_phi.data(), 16, "<c16", {N});
    writeNpy(out / "power_theta.npy", ff.power_theta.data(), 8, "<f8", {N});
    writeNpy(out / "power_phi.npy", ff.power_phi.data(), 8, "<f8", {N});
  }
  const NffftFd *nfd = dynamic_cast<const NffftFd *>(_nffft.get());
  if (nfd && !nfd->getOutputDirPath().empty() && !nfd->getTheta().empty() && !nfd->getPhi().empty()) {
    const std::filesystem::path out{nfd->getOutputDirPath()};
    if (!ensureDir(out)) return;
    const std::vector<size_t> shp{nfd->getFrequencies().size(), nfd->getTheta().size(), nfd->getPhi().size()};
    writeNpy(out / "frequencies.npy", nfd->getFrequencies().data(), 8, "<f8", {nfd->getFrequencies().size()});
    writeNpy(out / "theta.npy", nfd->getTheta().data(), 8, "<f8", {nfd->getTheta().size()});
    writeNpy(out / "phi.npy", nfd->getPhi().data(), 8, "<f8", {nfd->getPhi().size()});
    const char *names[8] = {"e_theta", "e_phi", "h_theta", "h_phi", "n_theta", "n_phi", "l_theta", "l_phi"};
    for (int w = 0; w < 8; ++w) {
      auto v = farField(w);
      writeNpy(out / (std::string(names[w]) + ".npy"), v.data(), 16, "<c16", shp);
    }
    auto p0 = farFieldPower(0), p1 = farFieldPower(1);
    writeNpy(out / "power_theta.npy", p0.data(), 8, "<f8", shp);
    writeNpy(out / "power_phi.npy", p1.data(), 8, "<f8", shp);
  }
}

void Simulation::checkRun(size_t total_time_steps) {
  init(total_time_steps);
  std::ofstream ofs{"simulation_check", std::ios::out};
  ofs << "nx:" << _nx << " ny:" << _ny << " nz:" << _nz << '\n';
  ofs << "Total size:" << _nx * _ny * _nz << '\n';
  std::ofstream object_ofs{"simulation_object_check", std::ios::out};
  object_ofs << "Object:" << '\n';
  for (auto &o : _objects) object_ofs << "Object: " << o->getName() << '\n';
}

}  // namespace xfdtd

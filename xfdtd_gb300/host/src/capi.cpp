// capi.cpp -- xfdtd_sim_* (include/xfdtd_sim.h): builds the C++ Simulation
// from a plain-C scene description and forwards to it.
#include <cstring>

#include "../../../include/xfdtd_sim.h"
#include "xfdtd/xfdtd.h"

struct xfdtd_sim {
  std::unique_ptr<xfdtd::Simulation> sim;
  std::vector<xfdtd::Monitor *> monitors;
  std::vector<std::shared_ptr<xfdtd::Monitor>> monitor_ptrs;
  std::shared_ptr<xfdtd::TFSF> tfsf;
  std::vector<double> nffft_freqs;
  int64_t nffft_box[3] = {0, 0, 0};
  std::string err;
};

namespace {

using namespace xfdtd;

// A Material of the description, or the dispersive medium it names.
// A plain material of the description (its eps_r from p[0] in double with
// XFDTD_MATERIAL_EXACT_EPS).
Material plainMaterial(const char *name, const xfdtd_material_desc &m) {
  if (m.flags & ~XFDTD_MATERIAL_EXACT_EPS) throw std::invalid_argument("unknown material flags");
  if (m.flags & XFDTD_MATERIAL_EXACT_EPS) {
    if (m.dispersion) throw std::invalid_argument("an exact eps_r is for plain materials only");
    return Material::withExactPermittivity(name, m.p[0], m.mu_r, m.sigma_e, m.sigma_m);
  }
  return Material(name, m.eps_r, m.mu_r, m.sigma_e, m.sigma_m);
}

std::unique_ptr<Material> makeMaterial(const xfdtd_material_desc &m) {
  switch (m.dispersion) {
    case XFDTD_DISPERSION_NONE:
      return std::make_unique<Material>(plainMaterial("material", m));
    case XFDTD_DISPERSION_LORENTZ:
      return std::make_unique<LorentzMedium>("lorentz", m.p[0], m.p[1], m.p[2], m.p[3], m.sigma_e, m.sigma_m);
    case XFDTD_DISPERSION_DRUDE:
      return std::make_unique<DrudeMedium>("drude", m.p[0], m.p[1], m.p[2], m.sigma_e, m.sigma_m);
    case XFDTD_DISPERSION_DEBYE:
      return std::make_unique<DebyMedium>("debye", m.p[0], m.p[1], m.p[2], m.sigma_e, m.sigma_m);
    default:
      throw std::invalid_argument("unknown dispersive medium kind");
  }
}

PointVector pv(const double *p) { return PointVector{p[0], p[1], p[2]}; }

std::unique_ptr<Shape> makeShape(const xfdtd_shape_desc &d) {
  switch (d.kind) {
    case XFDTD_SHAPE_CUBE: return std::make_unique<Cube>(pv(d.point), pv(d.size));
    case XFDTD_SHAPE_SPHERE: return std::make_unique<Sphere>(pv(d.point), d.radius);
    case XFDTD_SHAPE_CYLINDER:
      if (d.axis < 0 || d.axis > 2) throw std::invalid_argument("cylinder axis must be 0..2");
      return std::make_unique<Cylinder>(static_cast<Axis>(d.axis), pv(d.point), d.radius, d.height);
    default: throw std::invalid_argument("unknown shape kind");
  }
}

std::unique_ptr<Waveform> makeWaveform(const xfdtd_waveform_desc &w) {
  switch (w.kind) {
    case XFDTD_WAVE_GAUSSIAN: return std::make_unique<GaussianWaveform>(w.amplitude, w.tau, w.t0);
    case XFDTD_WAVE_COS_GAUSSIAN:
      return std::make_unique<CosineModulatedGaussianWaveform>(w.amplitude, w.tau, w.t0, w.frequency);
    case XFDTD_WAVE_SINUSOIDAL: return std::make_unique<SinusoidalWaveform>(w.amplitude, w.frequency, w.phase);
    case XFDTD_WAVE_CUSTOM: {
      if (!w.fn) throw std::invalid_argument("custom waveform without a callback");
      xfdtd_waveform_fn fn = w.fn;
      void *ctx = w.ctx;
      return std::make_unique<CustomWaveform>(w.amplitude, [fn, ctx](double t) { return fn(t, ctx); });
    }
    default: throw std::invalid_argument("unknown waveform kind");
  }
}

Orientation ori(int o) {
  if (o < 0 || o > 5) throw std::invalid_argument("orientation must be 0..5");
  return static_cast<Orientation>(o);
}
Axis axis(int a) {
  if (a < 0 || a > 2) throw std::invalid_argument("axis must be 0..2");
  return static_cast<Axis>(a);
}

template <class F>
int guarded(xfdtd_sim *s, F &&fn) {
  try {
    fn();
    return XFDTD_OK;
  } catch (const std::exception &e) {
    if (s) s->err = e.what();
    return XFDTD_ERR_INVALID_PLAN;
  }
}

}  // namespace

extern "C" {

int xfdtd_sim_create(const xfdtd_scene_desc *sc, int64_t total_steps, int precision, int flags, xfdtd_sim **out) {
  if (!sc || !out) return XFDTD_ERR_INVALID_PLAN;
  auto *s = new xfdtd_sim();
  *out = s;
  return guarded(s, [&] {
    auto sim = std::make_unique<Simulation>(sc->cell_size, sc->cfl);
    for (int i = 0; i < sc->n_objects; ++i) {
      const auto &o = sc->objects[i];
      if (o.kind == XFDTD_OBJECT_THIN_WIRE) {
        if (o.shape.kind != XFDTD_SHAPE_CYLINDER) throw std::runtime_error("ThinWire only support Cylinder shape");
        auto cy = std::make_unique<Cylinder>(axis(o.shape.axis), pv(o.shape.point), o.shape.radius, o.shape.height);
        sim->addObject(std::make_shared<ThinWire>("thin_wire", std::move(cy)));
      } else {
        sim->addObject(std::make_shared<Object>("object", makeShape(o.shape), makeMaterial(o.material)));
      }
    }
    for (int i = 0; i < sc->n_pml; ++i) {
      const auto &p = sc->pml[i];
      sim->addBoundary(std::make_shared<PML>(ori(p.orientation), p.thickness, p.order, p.sigma_ratio, p.alpha_min,
                                             p.alpha_max, p.kappa_max));
    }
    if (sc->tfsf.enabled) {
      const auto &t = sc->tfsf;
      std::shared_ptr<Waveform> w = makeWaveform(t.waveform);
      if (t.enabled == 2)   // TFSF2D(distance_x, distance_y, phi, e0, waveform)
        s->tfsf = std::make_shared<TFSF2D>(static_cast<SpatialIndex>(t.distance[0]),
                                           static_cast<SpatialIndex>(t.distance[1]), t.phi, t.e0, w);
      else
        s->tfsf = std::make_shared<TFSF3D>(static_cast<SpatialIndex>(t.distance[0]), static_cast<SpatialIndex>(t.distance[1]),
                                         static_cast<SpatialIndex>(t.distance[2]), t.e0, t.theta, t.phi, t.psi, w);
      sim->addTFSFSource(s->tfsf);
    }
    if (sc->nffft.enabled == 2) {   // NffftBroadBand(dx, dy, dz, theta, phi, path)
      const auto &n = sc->nffft;
      if (n.n_theta != 1 || n.n_phi != 1 || !n.theta || !n.phi)
        throw std::invalid_argument("a broadband NF-FF takes one theta and one phi");
      sim->addNFFFT(std::make_shared<NffftBroadBand>(static_cast<SpatialIndex>(n.distance[0]),
                                                     static_cast<SpatialIndex>(n.distance[1]),
                                                     static_cast<SpatialIndex>(n.distance[2]), n.theta[0], n.phi[0], ""));
      for (int a = 0; a < 3; ++a) s->nffft_box[a] = n.distance[a];
    } else if (sc->nffft.enabled) {
      const auto &n = sc->nffft;
      std::vector<double> f(n.frequencies, n.frequencies + n.n_freq);
      std::vector<double> th(n.theta, n.theta + n.n_theta), ph(n.phi, n.phi + n.n_phi);
      s->nffft_freqs = f;
      sim->addNFFFT(std::make_shared<NffftFd>(static_cast<SpatialIndex>(n.distance[0]),
                                              static_cast<SpatialIndex>(n.distance[1]),
                                              static_cast<SpatialIndex>(n.distance[2]), f, th, ph, ""));
      for (int a = 0; a < 3; ++a) s->nffft_box[a] = n.distance[a];
    }
    for (int i = 0; i < sc->n_lumped; ++i) {
      const auto &l = sc->lumped[i];
      auto cube = std::make_unique<Cube>(pv(l.point), pv(l.size));
      switch (l.kind) {
        case XFDTD_LUMPED_CURRENT_SOURCE:
          sim->addLumpedElement(std::make_shared<CurrentSource>(std::move(cube), ori(l.orientation), l.value,
                                                                makeWaveform(l.waveform)));
          break;
        case XFDTD_LUMPED_VOLTAGE_SOURCE:
          sim->addLumpedElement(std::make_shared<VoltageSource>(std::move(cube), ori(l.orientation), l.value,
                                                                makeWaveform(l.waveform)));
          break;
        case XFDTD_LUMPED_RESISTOR:
          sim->addLumpedElement(std::make_shared<Resistor>(std::move(cube), axis(l.orientation), l.value));
          break;
        case XFDTD_LUMPED_CAPACITOR:
          sim->addLumpedElement(std::make_shared<Capacitor>(std::move(cube), axis(l.orientation), l.value));
          break;
        case XFDTD_LUMPED_INDUCTOR:
          sim->addLumpedElement(std::make_shared<Inductor>(std::move(cube), axis(l.orientation), l.value));
          break;
        default: throw std::invalid_argument("unknown lumped element kind");
      }
    }
    for (int i = 0; i < sc->n_monitors; ++i) {
      const auto &m = sc->monitors[i];
      auto cube = std::make_unique<Cube>(pv(m.point), pv(m.size));
      std::shared_ptr<Monitor> mon;
      if (m.kind == XFDTD_MONITOR_VOLTAGE) {
        mon = std::make_shared<VoltageMonitor>(std::move(cube), ori(m.orientation), "", "");
      } else if (m.kind == XFDTD_MONITOR_CURRENT) {
        mon = std::make_shared<CurrentMonitor>(std::move(cube), ori(m.orientation), "", "");
      } else if (m.kind == XFDTD_MONITOR_FIELD) {
        if (m.component < 0 || m.component > 5 || m.plane_type < 0 || m.plane_type > 2)
          throw std::invalid_argument("bad field monitor component or plane type");
        auto fm = std::make_unique<TimeDomainFieldMonitor>(std::move(cube), static_cast<PlaneType>(m.plane_type),
                                                           static_cast<EMComponent>(m.component), "", "");
        if (m.plot_step > 0)
          mon = std::make_shared<MovieMonitor>(std::move(fm), static_cast<size_t>(m.total_time_steps),
                                               static_cast<size_t>(m.plot_step));
        else
          mon = std::move(fm);
      } else {
        throw std::invalid_argument("unknown monitor kind");
      }
      s->monitors.push_back(mon.get());
      s->monitor_ptrs.push_back(mon);
      sim->addMonitor(mon);
    }
    if (sc->n_ports > 0) {   // Network(ports, frequencies, output_path)
      if (!sc->ports || (sc->n_network_freqs > 0 && !sc->network_freqs)) throw std::invalid_argument("bad network");
      std::vector<std::unique_ptr<Port>> ports;
      for (int q = 0; q < sc->n_ports; ++q) {
        const auto &p = sc->ports[q];
        auto mon = [&](int m) {
          if (m < 0 || m >= static_cast<int>(s->monitor_ptrs.size())) throw std::invalid_argument("bad port monitor");
          return s->monitor_ptrs[m];
        };
        auto v = std::dynamic_pointer_cast<VoltageMonitor>(mon(p.voltage_monitor));
        auto c = std::dynamic_pointer_cast<CurrentMonitor>(mon(p.current_monitor));
        if (!v || !c) throw std::invalid_argument("a port takes a voltage monitor and a current monitor");
        ports.push_back(std::make_unique<Port>(p.index, std::complex<double>{p.impedance_re, p.impedance_im},
                                               p.is_activated_source != 0, v, c));
      }
      std::vector<double> fr(sc->network_freqs, sc->network_freqs + std::max(0, sc->n_network_freqs));
      sim->addNetwork(std::make_shared<Network>(std::move(ports), std::move(fr), ""));
    }
    if (sc->voxel_index) {
      std::vector<Material> mats;
      for (int q = 0; q < sc->n_voxel_materials; ++q) {
        const auto &m = sc->voxel_materials[q];
        if (m.dispersion) throw std::invalid_argument("voxel materials are plain materials (no dispersive media)");
        mats.push_back(plainMaterial("voxel", m));
      }
      const size_t cnt = static_cast<size_t>(sc->voxel_shape[0] * sc->voxel_shape[1] * sc->voxel_shape[2]);
      std::vector<uint32_t> idx(cnt);
      if (sc->voxel_index_bytes == 4) {
        const uint32_t *v = static_cast<const uint32_t *>(sc->voxel_index);
        std::copy(v, v + cnt, idx.begin());
      } else if (sc->voxel_index_bytes == 2 || sc->voxel_index_bytes == 0) {
        const uint16_t *v = static_cast<const uint16_t *>(sc->voxel_index);
        std::copy(v, v + cnt, idx.begin());
      } else {
        throw std::invalid_argument("voxel_index_bytes must be 2 or 4");
      }
      sim->setVoxelMaterials(std::move(mats), std::move(idx),
                             {static_cast<size_t>(sc->voxel_shape[0]), static_cast<size_t>(sc->voxel_shape[1]),
                              static_cast<size_t>(sc->voxel_shape[2])});
    }
    if (precision != XFDTD_FP64 && precision != XFDTD_FP32) throw std::invalid_argument("precision must be FP64 or FP32");
    sim->setPrecision(precision == XFDTD_FP64 ? Precision::FP64 : Precision::FP32);
    sim->setUseGraph((flags & XFDTD_FLAG_GRAPH) != 0);
    sim->setProfile((flags & XFDTD_FLAG_PROFILE) != 0);
    sim->setAutotune((flags & XFDTD_FLAG_AUTOTUNE) != 0);
    sim->setFusedSweep((flags & XFDTD_FLAG_FUSED_EH) ? 1 : (flags & XFDTD_FLAG_SPLIT_EH) ? 0 : -1);
    sim->setDevice((flags >> XFDTD_SIM_DEVICE_SHIFT) & 0xff);
    if (total_steps <= 0) throw std::invalid_argument("total_steps must be positive");
    sim->init(static_cast<size_t>(total_steps));
    s->sim = std::move(sim);
  });
}

int xfdtd_sim_step(xfdtd_sim *s, int64_t n) {
  if (!s || !s->sim) return XFDTD_ERR_STATE;
  return guarded(s, [&] {
    if (n < 0) throw std::invalid_argument("negative step count");
    s->sim->step(static_cast<size_t>(n));
  });
}

int xfdtd_sim_info(xfdtd_sim *s, int64_t out_n[3], double *out_dt, int64_t *out_step) {
  if (!s || !s->sim) return XFDTD_ERR_STATE;
  if (out_n) {
    out_n[0] = static_cast<int64_t>(s->sim->getNx());
    out_n[1] = static_cast<int64_t>(s->sim->getNy());
    out_n[2] = static_cast<int64_t>(s->sim->getNz());
  }
  if (out_dt) *out_dt = s->sim->getDt();
  if (out_step) *out_step = static_cast<int64_t>(s->sim->getCurrentTimeStep());
  return XFDTD_OK;
}

int xfdtd_sim_read_field(xfdtd_sim *s, int comp, double *out, int64_t len) {
  if (!s || !s->sim) return XFDTD_ERR_STATE;
  return guarded(s, [&] {
    auto v = s->sim->readField(comp);
    if (static_cast<size_t>(len) != v.size()) throw std::invalid_argument("length does not match the component");
    std::memcpy(out, v.data(), v.size() * sizeof(double));
  });
}

int xfdtd_sim_write_field(xfdtd_sim *s, int comp, const double *in, int64_t len) {
  if (!s || !s->sim) return XFDTD_ERR_STATE;
  return guarded(s, [&] { s->sim->writeField(comp, std::vector<double>(in, in + len)); });
}

int xfdtd_sim_read_monitor(xfdtd_sim *s, int index, double *out, int64_t len) {
  if (!s || !s->sim) return XFDTD_ERR_STATE;
  return guarded(s, [&] {
    const size_t total = s->sim->getTotalTimeSteps();
    if (index < 0 || index >= static_cast<int>(s->monitors.size())) throw std::invalid_argument("bad monitor index");
    if (static_cast<size_t>(len) != total) throw std::invalid_argument("length must be total_steps");
    const auto v = s->sim->monitorValues(static_cast<size_t>(index));
    std::memcpy(out, v.data(), total * sizeof(double));
  });
}

int xfdtd_sim_field_monitor(xfdtd_sim *s, int index, int64_t lo[3], int64_t shape[3], int64_t *n_frames,
                            int64_t *steps, int64_t max) {
  if (!s || !s->sim) return XFDTD_ERR_STATE;
  return guarded(s, [&] {
    if (index < 0 || index >= static_cast<int>(s->monitors.size())) throw std::invalid_argument("bad monitor index");
    const auto shp = s->sim->fieldMonitorShape(static_cast<size_t>(index));
    const auto first = s->sim->fieldMonitorOrigin(static_cast<size_t>(index));
    if (lo)
      for (int a = 0; a < 3; ++a) lo[a] = static_cast<int64_t>(first[a]);
    const auto st = s->sim->fieldMonitorSteps(static_cast<size_t>(index));
    if (shape)
      for (int a = 0; a < 3; ++a) shape[a] = static_cast<int64_t>(shp[a]);
    if (n_frames) *n_frames = static_cast<int64_t>(st.size());
    if (steps)
      for (size_t f = 0; f < st.size() && static_cast<int64_t>(f) < max; ++f) steps[f] = st[f];
  });
}

int xfdtd_sim_read_field_monitor(xfdtd_sim *s, int index, int64_t frame, double *out, int64_t len) {
  if (!s || !s->sim || !out) return XFDTD_ERR_STATE;
  return guarded(s, [&] {
    if (index < 0 || index >= static_cast<int>(s->monitors.size())) throw std::invalid_argument("bad monitor index");
    if (frame < 0) throw std::invalid_argument("bad frame");
    const auto v = s->sim->fieldMonitorFrame(static_cast<size_t>(index), static_cast<size_t>(frame));
    if (static_cast<size_t>(len) != v.size()) throw std::invalid_argument("length must be the monitor's box cells");
    std::memcpy(out, v.data(), v.size() * sizeof(double));
  });
}

int xfdtd_sim_read_nffft(xfdtd_sim *s, int which, double *out, int64_t len) {
  if (!s || !s->sim) return XFDTD_ERR_STATE;
  return guarded(s, [&] {
    auto v = s->sim->nffftAccumulator(which);
    if (static_cast<size_t>(len) != 2 * v.size()) throw std::invalid_argument("length mismatch");
    std::memcpy(out, v.data(), v.size() * sizeof(std::complex<double>));
  });
}

int xfdtd_sim_far_field(xfdtd_sim *s, int which, double *out, int64_t len) {
  if (!s || !s->sim) return XFDTD_ERR_STATE;
  return guarded(s, [&] {
    if (dynamic_cast<const NffftBroadBand *>(s->sim->getNFFFT())) {
      const auto ff = s->sim->broadbandFarField();
      const std::vector<std::complex<double>> *cx[8] = {&ff.e_theta, &ff.e_phi, &ff.h_theta, &ff.h_phi,
                                                       &ff.n_theta, &ff.n_phi, &ff.l_theta, &ff.l_phi};
      const std::vector<double> *re[3] = {&ff.power_theta, &ff.power_phi, &ff.frequencies};
      if (which >= 0 && which < 8) {
        if (static_cast<size_t>(len) != 2 * cx[which]->size()) throw std::invalid_argument("length mismatch");
        std::memcpy(out, cx[which]->data(), cx[which]->size() * sizeof(std::complex<double>));
      } else if (which >= 8 && which <= 10) {
        if (static_cast<size_t>(len) != re[which - 8]->size()) throw std::invalid_argument("length mismatch");
        std::memcpy(out, re[which - 8]->data(), re[which - 8]->size() * sizeof(double));
      } else {
        throw std::invalid_argument("broadband far-field output must be 0..10");
      }
      return;
    }
    if (which >= 0 && which < 8) {
      auto v = s->sim->farField(which);
      if (static_cast<size_t>(len) != 2 * v.size()) throw std::invalid_argument("length mismatch");
      std::memcpy(out, v.data(), v.size() * sizeof(std::complex<double>));
    } else if (which == 8 || which == 9) {
      auto v = s->sim->farFieldPower(which - 8);
      if (static_cast<size_t>(len) != v.size()) throw std::invalid_argument("length mismatch");
      std::memcpy(out, v.data(), v.size() * sizeof(double));
    } else {
      throw std::invalid_argument("far-field output must be 0..9");
    }
  });
}

int xfdtd_sim_incident_dft(xfdtd_sim *s, const double *freqs, int n, double *out) {
  if (!s || !s->sim) return XFDTD_ERR_STATE;
  return guarded(s, [&] {
    if (!s->tfsf) throw std::runtime_error("no TFSF source");
    auto r = s->tfsf->getIncidentWaveFourierTransform(std::vector<double>(freqs, freqs + n));
    for (int i = 0; i < n; ++i) {
      out[2 * i] = r[i].real();
      out[2 * i + 1] = r[i].imag();
    }
  });
}

int xfdtd_sim_s_parameters(xfdtd_sim *s, int32_t *keys, int64_t max, int64_t *count, int64_t *n_freq) {
  if (!s || !s->sim) return XFDTD_ERR_STATE;
  return guarded(s, [&] {
    const auto &sp = s->sim->sParameters();
    if (count) *count = static_cast<int64_t>(sp.size());
    if (n_freq) *n_freq = static_cast<int64_t>(s->sim->getNetwork()->getFrequencies().size());
    int64_t q = 0;
    for (const auto &e : sp) {
      if (keys && q < max) keys[q] = e.first;
      ++q;
    }
  });
}

int xfdtd_sim_read_s_parameter(xfdtd_sim *s, int key, double *out, int64_t len) {
  if (!s || !s->sim || !out) return XFDTD_ERR_STATE;
  return guarded(s, [&] {
    const auto &sp = s->sim->sParameters();
    auto it = sp.find(key);
    if (it == sp.end()) throw std::invalid_argument("no such S-parameter");
    if (static_cast<size_t>(len) != 2 * it->second.size()) throw std::invalid_argument("length must be 2 * n_freq");
    std::memcpy(out, it->second.data(), it->second.size() * sizeof(std::complex<double>));
  });
}

int xfdtd_sim_set_output(xfdtd_sim *s, int index, const char *dir, const char *file) {
  if (!s || !s->sim) return XFDTD_ERR_STATE;
  return guarded(s, [&] {
    if (index == -2) {
      if (!s->sim->getNetwork()) throw std::invalid_argument("no network in this simulation");
      s->sim->getNetwork()->setOutputPath(dir ? dir : "");
      return;
    }
    if (index == -1) {
      if (!s->sim->getNFFFT()) throw std::invalid_argument("no NF-FF in this simulation");
      s->sim->getNFFFT()->setOutputDirPath(dir ? dir : "");
      return;
    }
    if (index < 0 || index >= static_cast<int>(s->monitors.size())) throw std::invalid_argument("bad monitor index");
    s->monitors[index]->setOutputDirPath(dir ? dir : "");
    s->monitors[index]->setOutputFileName(file ? file : "");
  });
}

int xfdtd_sim_output(xfdtd_sim *s) {
  if (!s || !s->sim) return XFDTD_ERR_STATE;
  return guarded(s, [&] { s->sim->outputData(); });
}

xfdtd_handle *xfdtd_sim_engine(xfdtd_sim *s) { return (s && s->sim) ? s->sim->engine() : nullptr; }

const char *xfdtd_sim_last_error(xfdtd_sim *s) { return s ? s->err.c_str() : "null simulation"; }

void xfdtd_sim_destroy(xfdtd_sim *s) { delete s; }

}  // extern "C"

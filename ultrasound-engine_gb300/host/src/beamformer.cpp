// beamformer.cpp — host front end of the GPU beamformer (behaviour of the
// reference's core/src/beamformer.cpp:218-569). A Beamformer keeps a small
// cache of device plans (channel metadata, grid and config frozen on the GPU)
// so that repeated frames with the same geometry pay only for the transfer of
// their samples and the kernels.
#include "usx/beamformer.hpp"

#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <list>
#include <map>
#include <mutex>
#include <set>
#include <stdexcept>

#include "desc.hpp"
#include "usx/geometry.hpp"
#include "usx/runtime.hpp"

namespace usx {

void BeamformerConfig::validate() const {
  if (f_number <= 0) throw std::invalid_argument("BeamformerConfig.f_number must be > 0");
  if (mv_subarray < 2) throw std::invalid_argument("BeamformerConfig.mv_subarray must be >= 2");
  if (mv_diagonal_loading < 0)
    throw std::invalid_argument("BeamformerConfig.mv_diagonal_loading must be >= 0");
  if (mv_range_average < 0)
    throw std::invalid_argument("BeamformerConfig.mv_range_average must be >= 0");
}

namespace {

// The learned minimum-variance network of a context: read once from
// USX_LEARNED_MV_WEIGHTS, else the weights shipped beside the library
// (<package>/weights/learned_mv_128ch_l64.bin), with the gates and subspace
// refinement recorded in the ".gate" file written with the weights
// ("<gate> [<beams> [<share gate> [<level gate>]]]"); without it, gate 0.05,
// no refinement and no share or level gate. BeamformerConfig's learned_* fields override these per
// beamformer. The weights file is the trainer's raw format: "USXMLP1\0",
// int32 n_layers, int32 dims[n_layers + 1], float32 parameters.
struct LearnedNet {
  usx_mlp* mlp = nullptr;
  float gate = 0.05f;
  int refine = -1;   // DFT beams of the subspace refinement (< 0: none)
  float share_gate = INFINITY;
  float level_gate = INFINITY;
  int level_lines = 0, level_depths = 0;  // the level gate's neighbourhood
};

std::string library_dir() {
  Dl_info info{};
  if (dladdr(reinterpret_cast<void*>(&library_dir), &info) && info.dli_fname) {
    std::string p(info.dli_fname);
    const auto k = p.find_last_of('/');
    if (k != std::string::npos) return p.substr(0, k);
  }
  return ".";
}

LearnedNet learned_net(usx_ctx* ctx) {
  static std::mutex mu;
  static std::map<usx_ctx*, LearnedNet> nets;
  std::lock_guard<std::mutex> lock(mu);
  auto it = nets.find(ctx);
  if (it != nets.end()) return it->second;
  const char* env = std::getenv("USX_LEARNED_MV_WEIGHTS");
  const std::string path = env ? std::string(env) : library_dir() + "/../weights/learned_mv_128ch_l64.bin";
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("learned minimum variance: cannot open the network weights " + path);
  char magic[8];
  std::int32_t n_layers = 0;
  f.read(magic, 8);
  f.read(reinterpret_cast<char*>(&n_layers), 4);
  if (!f || std::memcmp(magic, "USXMLP1\0", 8) != 0 || n_layers < 1 || n_layers > 64)
    throw std::runtime_error("learned minimum variance: " + path + " is not a network file");
  std::vector<int> dims(static_cast<std::size_t>(n_layers) + 1);
  f.read(reinterpret_cast<char*>(dims.data()), 4 * static_cast<std::streamsize>(dims.size()));
  std::size_t n_params = 0;
  for (int l = 0; l < n_layers; ++l)
    n_params += static_cast<std::size_t>(dims[l]) * dims[l + 1] + static_cast<std::size_t>(dims[l + 1]);
  std::vector<float> params(n_params);
  f.read(reinterpret_cast<char*>(params.data()), static_cast<std::streamsize>(4 * n_params));
  if (!f) throw std::runtime_error("learned minimum variance: " + path + " is truncated");
  LearnedNet net;
  rt::check(usx_cu_mlp_create(ctx, n_layers, dims.data(), 0, &net.mlp), "learned network");
  rt::check(usx_cu_mlp_set_params(net.mlp, params.data()), "learned network weights");
  {
    // "<gate> [<refine beams> [<share gate> [<level gate>]]]", as written by the trainer's evaluation.
    std::ifstream gf(path.substr(0, path.size() - 4) + ".gate");
    std::string gs;
    if (gf >> gs) net.gate = std::strtof(gs.c_str(), nullptr);
    int rv = 0;
    if (gf >> rv) net.refine = rv;
    if (gf >> gs) net.share_gate = std::strtof(gs.c_str(), nullptr);
    if (gf >> gs) net.level_gate = std::strtof(gs.c_str(), nullptr);
    if (gf >> gs) net.level_lines = std::atoi(gs.c_str());
    if (gf >> gs) net.level_depths = std::atoi(gs.c_str());
  }
  nets.emplace(ctx, net);
  return net;
}

}  // namespace

// The key of a plan is everything that is frozen into it. The grid's points
// (6 MB for 512 x 1024 pixels) are compared in place, not copied, on every
// lookup; only a new plan keeps a copy.
struct PlanKey {
  usx_ctx* ctx = nullptr;
  std::vector<unsigned char> meta;   // POD bytes of probe/medium/acq/config/tx geometry
  std::vector<real> points;
  bool matches(usx_ctx* c, const std::vector<unsigned char>& m, const real* pts, std::size_t n) const {
    return ctx == c && meta == m && points.size() == n &&
           (n == 0 || std::memcmp(points.data(), pts, n * sizeof(real)) == 0);
  }
};

class PlanCache {
 public:
  ~PlanCache() {
    for (auto& e : entries_) usx_cu_bf_plan_destroy(e.second);
  }
  usx_bf_plan* get(const ChannelData& data, const ScanGrid& grid, const BeamformerConfig& cfg,
                   int ev_begin, int ev_end) {
    PlanKey key;
    key.ctx = rt::ctx();
    const usx_probe p = desc::probe(data.probe);
    const usx_medium m = desc::medium(data.medium);
    const usx_acquisition a = desc::acq(data.acq);
    const usx_beamformer_config b = desc::bf(cfg);
    auto put = [&](const void* x, std::size_t n) {
      const auto* c = static_cast<const unsigned char*>(x);
      key.meta.insert(key.meta.end(), c, c + n);
    };
    put(&p, sizeof p);
    put(&m, sizeof m);
    put(&a, sizeof a);
    put(&b, sizeof b);
    const int iq = data.is_iq ? 1 : 0;
    put(&iq, sizeof iq);
    // Settings frozen into the plan that the C descriptor does not carry.
    const int solver = static_cast<int>(cfg.mv_solver);
    put(&solver, sizeof solver);
    put(&cfg.learned_gate, sizeof(real));
    put(&cfg.learned_refine, sizeof(int));
    put(&cfg.learned_share_gate, sizeof(real));
    put(&cfg.learned_level_gate, sizeof(real));
    put(&data.demodulation_frequency, sizeof(real));
    put(&ev_begin, sizeof ev_begin);
    put(&ev_end, sizeof ev_end);
    const int gt = static_cast<int>(grid.type);
    put(&gt, sizeof gt);
    put(&grid.n_axis0, sizeof(int));
    put(&grid.n_axis1, sizeof(int));
    for (const Transmit& t : data.transmits) {
      const int ty = static_cast<int>(t.type);
      put(&ty, sizeof ty);
      put(&t.angle, sizeof(real));
      put(&t.focus, sizeof(Vec3));
      put(&t.origin, sizeof(Vec3));
      const int na = static_cast<int>(t.apodization.size());
      put(&na, sizeof na);
      if (na) put(t.apodization.data(), sizeof(real) * t.apodization.size());
    }
    const real* pts = desc::points(grid);
    const std::size_t n_pts = 3 * grid.points.size();

    std::lock_guard<std::mutex> lock(mu_);
    for (auto it = entries_.begin(); it != entries_.end(); ++it) {
      if (it->first.matches(key.ctx, key.meta, pts, n_pts)) {
        entries_.splice(entries_.begin(), entries_, it);
        return entries_.front().second;
      }
    }
    key.points.assign(pts, pts + n_pts);
    desc::Channel ch(data);
    const usx_grid_desc g = desc::grid(grid);
    usx_bf_plan* plan = nullptr;
    rt::check(usx_cu_bf_plan_create(key.ctx, &ch.cd, &g, desc::points(grid), &b, ev_begin, ev_end, &plan),
              "beamformer plan");
    // Minimum variance runs on the tensor cores (BF16 covariance, FP32
    // refinement, FP64 re-solve where needed) unless the config asks for the
    // reference's FP32 operation order.
    if (cfg.combiner == Combiner::MV && cfg.mv_solver == MvSolver::Tensor)
      usx_cu_bf_plan_set_mv_mode(plan, USX_MV_TENSOR);  // unsupported shapes stay exact
    if ((cfg.combiner == Combiner::MV || cfg.combiner == Combiner::LearnedMV) && cfg.mv_solver == MvSolver::FP32)
      usx_cu_bf_plan_set_mv_mode(plan, USX_MV_FP32);
    if (cfg.combiner == Combiner::LearnedMV) {
      try {
        const LearnedNet net = learned_net(key.ctx);
        const float gate = cfg.learned_gate >= 0.0f ? cfg.learned_gate : net.gate;
        const int refine = cfg.learned_refine != -2 ? cfg.learned_refine : net.refine;
        const float share = cfg.learned_share_gate >= 0.0f ? cfg.learned_share_gate : net.share_gate;
        rt::check(usx_cu_bf_plan_set_learned(plan, net.mlp, gate), "learned minimum variance");
        rt::check(usx_cu_bf_plan_set_learned_refine(plan, refine), "learned minimum variance refinement");
        rt::check(usx_cu_bf_plan_set_learned_subspace(plan, 1, share), "learned minimum variance share gate");
        const float level = cfg.learned_level_gate >= 0.0f ? cfg.learned_level_gate : net.level_gate;
        rt::check(usx_cu_bf_plan_set_learned_level_gate(plan, level), "learned minimum variance level gate");
        rt::check(usx_cu_bf_plan_set_learned_level_window(plan, net.level_lines, net.level_depths),
                  "learned minimum variance level window");
      } catch (...) {
        usx_cu_bf_plan_destroy(plan);
        throw;
      }
    }
    entries_.emplace_front(std::move(key), plan);
    while (entries_.size() > kMaxPlans) {
      used_.erase(entries_.back().second);
      usx_cu_bf_plan_destroy(entries_.back().second);
      entries_.pop_back();
    }
    return plan;
  }

  // True the first time it is asked about `plan` (the plan was just created).
  bool first_use(usx_bf_plan* plan) {
    std::lock_guard<std::mutex> lock(mu_);
    return used_.insert(plan).second;
  }

 private:
  static constexpr std::size_t kMaxPlans = 4;
  std::mutex mu_;
  std::list<std::pair<PlanKey, usx_bf_plan*>> entries_;
  std::set<usx_bf_plan*> used_;
};

// (pixels x events x channels) above which a new plan autotunes on its first frame.
constexpr double kAutotuneWork = 1e9;

Beamformer::Beamformer(BeamformerConfig config) : config_(config), plans_(std::make_shared<PlanCache>()) {
  config_.validate();
}
Beamformer::~Beamformer() = default;
Beamformer::Beamformer(const Beamformer& o) : config_(o.config_), plans_(std::make_shared<PlanCache>()) {}
Beamformer& Beamformer::operator=(const Beamformer& o) {
  config_ = o.config_;
  plans_ = std::make_shared<PlanCache>();
  return *this;
}

namespace {
const void* upload(const ChannelData& data) {
  if (data.is_iq) {
    if (data.iq.size() != data.size()) throw std::invalid_argument("ChannelData has no IQ samples");
    void* d = rt::slot(3, data.iq.size() * sizeof(cplx));
    rt::h2d(d, data.iq.data(), data.iq.size() * sizeof(cplx));
    return d;
  }
  if (data.rf.size() != data.size()) throw std::invalid_argument("ChannelData has no RF samples");
  void* d = rt::slot(3, data.rf.size() * sizeof(float));
  rt::h2d(d, data.rf.data(), data.rf.size() * sizeof(float));
  return d;
}
}  // namespace

Frame Beamformer::beamform(const ChannelData& data, const ScanGrid& grid, int event_begin,
                           int event_end) const {
  data.validate();
  grid.validate();
  config_.validate();
  return beamform_device(data, upload(data), grid, event_begin, event_end);
}

void Beamformer::beamform_into(const ChannelData& data, const void* d_in, const ScanGrid& grid, void* d_out,
                               int event_begin, int event_end) const {
  data.validate();
  grid.validate();
  config_.validate();
  const int n_ev = data.n_events();
  if (event_end < 0) event_end = n_ev;
  event_begin = std::clamp(event_begin, 0, n_ev);
  event_end = std::clamp(event_end, event_begin, n_ev);
  usx_bf_plan* plan = plans_->get(data, grid, config_, event_begin, event_end);
  // A plan's first frame of a large acquisition picks the delay-and-sum launch
  // shape by timing each variant on it (the frame is the chosen variant's).
  const double work = static_cast<double>(grid.n_pixels()) * (event_end - event_begin) * data.n_channels();
  if (work >= kAutotuneWork && plans_->first_use(plan))
    rt::check(usx_cu_bf_plan_autotune(plan, d_in, static_cast<float*>(d_out), 1, nullptr), "beamform autotune");
  else
    rt::check(usx_cu_bf_execute(plan, d_in, static_cast<float*>(d_out)), "beamform");
}

Frame Beamformer::beamform_device(const ChannelData& data, const void* d_in, const ScanGrid& grid,
                                  int event_begin, int event_end) const {
  Frame frame;
  frame.grid = grid;
  frame.demodulation_frequency = data.is_iq ? data.demodulation_frequency : 0.0f;
  frame.allocate();
  void* d_out = rt::slot(4, frame.data.size() * sizeof(cplx));
  beamform_into(data, d_in, grid, d_out, event_begin, event_end);
  rt::d2h(frame.data.data(), d_out, frame.data.size() * sizeof(cplx));
  return frame;
}

std::vector<Frame> Beamformer::beamform_sequence(const ChannelData& data, const ScanGrid& grid,
                                                 int events_per_frame) const {
  if (events_per_frame <= 0)
    throw std::invalid_argument("beamform_sequence: events_per_frame must be > 0");
  data.validate();
  grid.validate();
  config_.validate();
  const int n_ev = data.n_events();
  const int n_frames = n_ev / events_per_frame;
  if (n_frames == 0) throw std::invalid_argument("beamform_sequence: fewer events than events_per_frame");
  usx_bf_plan* plan = plans_->get(data, grid, config_, 0, n_ev);
  const void* d_in = upload(data);
  const std::size_t n_pix = static_cast<std::size_t>(grid.n_pixels());
  void* d_out = rt::slot(4, n_pix * n_frames * sizeof(cplx));
  rt::check(usx_cu_bf_execute_sequence(plan, events_per_frame, n_frames, d_in,
                                       static_cast<float*>(d_out), static_cast<int64_t>(n_pix)),
            "beamform_sequence");
  std::vector<Frame> frames(static_cast<std::size_t>(n_frames));
  std::vector<cplx> all(n_pix * n_frames);
  rt::d2h(all.data(), d_out, all.size() * sizeof(cplx));
  for (int f = 0; f < n_frames; ++f) {
    Frame& fr = frames[static_cast<std::size_t>(f)];
    fr.grid = grid;
    fr.demodulation_frequency = data.is_iq ? data.demodulation_frequency : 0.0f;
    fr.data.assign(all.begin() + static_cast<std::ptrdiff_t>(n_pix * f),
                   all.begin() + static_cast<std::ptrdiff_t>(n_pix * (f + 1)));
    fr.sequence = f;
    fr.timestamp = static_cast<double>(f) * events_per_frame / data.acq.prf;
  }
  return frames;
}

real transmit_sensitivity(const Probe& probe, const Transmit& tx, const Vec3& point, real wavelength) {
  // Scalar restatement of the illumination weight (beamformer.cpp:238-295).
  bool valid = false;
  real x_lo = 0, x_hi = 0;
  for (int i = 0; i < probe.n_elements; ++i) {
    if (!tx.apodization.empty() && tx.apodization[static_cast<std::size_t>(i)] == 0.0f) continue;
    const real x = probe.element_position(i).x;
    if (!valid) { x_lo = x_hi = x; valid = true; }
    else { x_lo = std::min(x_lo, x); x_hi = std::max(x_hi, x); }
  }
  if (!valid || point.z <= 0.0f) return 0.0f;
  real a, b;
  if (tx.type == TransmitType::PlaneWave) {
    const real shift = point.z * std::tan(tx.angle);
    a = x_lo + shift;
    b = x_hi + shift;
  } else {
    const real zf = tx.focus.z;
    if (std::abs(zf) < 1e-9f) return 1.0f;
    a = x_lo + (tx.focus.x - x_lo) * point.z / zf;
    b = x_hi + (tx.focus.x - x_hi) * point.z / zf;
    if (a > b) std::swap(a, b);
  }
  const real aperture = std::max(x_hi - x_lo, probe.pitch);
  const real diffraction = std::clamp(point.z / aperture, 0.5f, 20.0f) * wavelength;
  a -= diffraction;
  b += diffraction;
  const real centre = 0.5f * (a + b), half = 0.5f * (b - a);
  if (half <= 0.0f) return 0.0f;
  return window_value(Window::Tukey, (point.x - centre) / half, 0.4f);
}

}  // namespace usx

// Host driver for the GB300 path: the reference's driver loop (app/main.cpp:20-56
// with app/simulation_configuration.h) selected by `compute_type=gb300`, running
// the pre-loop and main loop through the C ABI of include/sphg.h.
// compute_type=sorted is an alias of gb300; lists and mp-lists select the
// library's lists compute mode (CSR lists assembled every iteration).
//
// Unchanged from the reference, so an existing run directory works as is:
//   * the configuration file and its keys (config/example.txt; parser semantics
//     of core/utils/InputParser.cpp:10-31: `key = value` lines, values trimmed of
//     blanks and tabs, a missing key reads as "0");
//   * the domain [0, domain_x] x [0, domain_y] (app/simulation_configuration.h:80-87)
//     and the lattice (LatticeCreator::CreateLattice, core/container/Lattice.h:12-35:
//     ceil(vol*L/d)+1 points per direction at d*i, index i + nx*j);
//   * the step sequence (PreLoopComputation / MainLoopComputation,
//     app/simulation_configuration.h:183-400): step 0 is the pre-loop, steps
//     1..steps-1 each integrate, re-sort, and compute density, pressure, forces;
//   * the checkpoint files positions_step_<i>.txt, "x y z" per particle in the
//     current (cell-sorted) order with the stream's default formatting
//     (core/utils/CheckPointWriter.cpp:11-27), written every
//     checkpoint_write_frequency steps and for step 0 if bool_output_first_step;
//   * the step header "Step= i\t N=..\t E_k=..\t |v|_max=..", |v|_max being the
//     maximum SQUARED speed (app/simulation_configuration.h:152-158,
//     core/container/MeasuringFunctions.h:5-61);
//   * cells_<i>.txt ("cell:c[start,end)", -1 for an empty cell) when
//     bool_measure_neighborhood is set (app/simulation_configuration.h:34-45),
//     and then also one line of neighbour and cell statistics of the last
//     iteration in neighborhood_and_cells.data (AvgNeighborsPerParticle,
//     core/algorithmic/MeasureAverageNeighborsPerParticle.h);
//   * the timer summary on stdout and one appended line in timer_manager.data
//     (core/utils/TimerManager.cpp:3-40).
//
// Keys the reference fixes at compile time (core/ConfigVariables.hpp:9-14) are
// read from the file, with the reference's values as defaults: H (1),
// GAS_CONSTANT (30), RHO_0 (25), MU (0.01).  Library extensions, all optional:
// gravity_x (0), gravity_y (-10), mass (1), alpha (0), c0 (0), periodic (0),
// precision (plain|split), use_graph (1), header_frequency (1), output_dir (.),
// snapshot_write_frequency (0 = never), snapshot_prefix (snapshot_step_),
// resume_from (a snapshot file; the run continues after its step).
//
// Checkpoints are formatted and written by a background thread from a small
// pool of host buffers, so the GPU keeps stepping while a file is written.
//
// `--dry-run` parses the configuration, builds the lattice, prints the
// configuration and exits without touching the GPU.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "sphg.h"

namespace {

// ---- configuration file (core/utils/InputParser.cpp:10-31) ------------------
std::string trim(const std::string& s) {
  const size_t a = s.find_first_not_of(" \t\r");
  const size_t b = s.find_last_not_of(" \t\r");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

struct Config {
  std::map<std::string, std::string> kv;

  bool read(const std::string& path) {
    std::ifstream f(path);
    if (!f.is_open()) return false;
    std::string line;
    while (std::getline(f, line)) {
      const size_t eq = line.find('=');
      if (eq == std::string::npos) continue;
      // first occurrence wins, as std::map::insert does in the reference
      kv.insert({trim(line.substr(0, eq)), trim(line.substr(eq + 1))});
    }
    return true;
  }
  bool has(const char* k) const { return kv.count(k) != 0; }
  std::string str(const char* k, const char* def = "0") const {
    auto it = kv.find(k);
    return it == kv.end() ? std::string(def) : it->second;
  }
  double real(const char* k, double def = 0.0) const { return has(k) ? std::stod(str(k)) : def; }
  long long integer(const char* k, long long def = 0) const { return has(k) ? std::stoll(str(k)) : def; }
  bool boolean(const char* k) const {  // istream >> bool: "1" true, anything else false
    bool b = false;
    std::istringstream(str(k)) >> b;
    return b;
  }
};

// ---- timers (core/utils/TimerManager.cpp) ------------------------------------
struct Timers {
  using clock = std::chrono::steady_clock;
  std::vector<std::string> names;
  std::map<std::string, double> total;
  std::map<std::string, clock::time_point> start_at;
  void add(const std::string& n) {
    names.push_back(n);
    total[n] = 0.0;
  }
  void start(const std::string& n) { start_at[n] = clock::now(); }
  void stop(const std::string& n) {
    total[n] += std::chrono::duration<double>(clock::now() - start_at[n]).count();
  }
  void print() const {
    double sum = 0.0;
    std::cout << "[HighPerformanceClock] Measured times: \n";
    for (const auto& n : names) {
      std::cout << n << "=" << total.at(n) << "\n";
      sum += total.at(n);
    }
    std::cout << "Total time=" << sum - total.at("main_loop") << "\n";
  }
  void append_file(const std::string& path, long long steps, long long n) const {
    const bool fresh = !std::ifstream(path).good();
    std::ofstream f(path, std::ios::app);
    if (!f) return;
    if (fresh) {
      f << std::fixed << std::setw(20) << std::left << "#threads" << "\t" << std::setw(20) << "#steps"
        << "\t" << std::setw(20) << "N" << "\t";
      for (const auto& nm : names) f << std::setw(20) << std::left << nm << "\t";
      f << std::endl;
    }
    f << std::fixed << std::setw(20) << std::left << 1 << "\t" << std::setw(20) << steps << "\t"
      << std::setw(20) << n << "\t";
    for (const auto& nm : names) f << std::setw(20) << std::setprecision(8) << std::left << total.at(nm) << "\t";
    f << std::endl;
  }
};

// ---- asynchronous checkpoint writer (core/utils/CheckPointWriter.cpp:11-27) --
class CheckpointWriter {
 public:
  CheckpointWriter(std::string prefix, size_t n, int pool = 3) : prefix_(std::move(prefix)) {
    for (int i = 0; i < pool; ++i) free_.push_back(new Buf{-1, std::vector<double>(n), std::vector<double>(n)});
    worker_ = std::thread([this] { run(); });
  }
  ~CheckpointWriter() { finish(); }
  struct Buf {
    long long step;
    std::vector<double> x, y;
  };
  // A free buffer (blocks while all are queued for writing).
  Buf* acquire() {
    std::unique_lock<std::mutex> lk(m_);
    cv_.wait(lk, [this] { return !free_.empty(); });
    Buf* b = free_.front();
    free_.pop_front();
    return b;
  }
  void submit(Buf* b) {
    {
      std::lock_guard<std::mutex> lk(m_);
      todo_.push_back(b);
    }
    cv_.notify_all();
  }
  void finish() {
    if (!worker_.joinable()) return;
    {
      std::lock_guard<std::mutex> lk(m_);
      done_ = true;
    }
    cv_.notify_all();
    worker_.join();
    for (Buf* b : free_) delete b;
    free_.clear();
  }
  bool failed() const { return failed_; }

 private:
  void run() {
    std::vector<char> text;
    for (;;) {
      Buf* b = nullptr;
      {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [this] { return done_ || !todo_.empty(); });
        if (todo_.empty()) return;
        b = todo_.front();
        todo_.pop_front();
      }
      write(*b);
      {
        std::lock_guard<std::mutex> lk(m_);
        free_.push_back(b);
      }
      cv_.notify_all();
    }
  }
  void write(const Buf& b) {
    const std::string name = prefix_ + std::to_string(b.step) + ".txt";
    FILE* f = std::fopen(name.c_str(), "w");
    if (!f) {
      failed_ = true;
      return;
    }
    std::vector<char> out;
    out.reserve(b.x.size() * 28);
    char line[96];
    for (size_t i = 0; i < b.x.size(); ++i) {
      // operator<< on a double with default flags and precision 6 is %g
      const int len = std::snprintf(line, sizeof(line), "%g %g %g\n", b.x[i], b.y[i], 0.0);
      out.insert(out.end(), line, line + len);
    }
    if (std::fwrite(out.data(), 1, out.size(), f) != out.size()) failed_ = true;
    std::fclose(f);
  }

  std::string prefix_;
  std::mutex m_;
  std::condition_variable cv_;
  std::deque<Buf*> free_, todo_;
  bool done_ = false;
  bool failed_ = false;
  std::thread worker_;
};

void die(const char* what, sphg_status st) {
  std::cerr << "[Error] " << what << ": status " << (int)st << ": " << sphg_last_error_string() << std::endl;
  std::exit(1);
}

int next_pow2(int v) {
  int p = 1;
  while (p < v) p *= 2;
  return p;
}

uint32_t morton2(uint32_t x, uint32_t y) {
  auto spread = [](uint32_t v) {
    v &= 0x0000ffffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
  };
  return spread(x) | (spread(y) << 1);
}

}  // namespace

int main(int argc, char** argv) {
  std::string path = "example.txt";
  bool dry = false;
  for (int i = 1; i < argc; ++i) {
    if (std::strcmp(argv[i], "--dry-run") == 0)
      dry = true;
    else
      path = argv[i];
  }
  std::cout << "[Smoothed Particle Hydrodynamics]\n";
  Config cfg;
  if (!cfg.read(path)) {
    std::cerr << "[Error]Cannot find configuration file " << path << std::endl;
    return 1;
  }
  Timers timers;
  for (const char* n : {"main_loop", "gpu_step", "neighbor_list", "cuda_buffer_copy", "IO"}) timers.add(n);
  std::cout << "[Build] Using GB300 acceleration (libsphg " << sphg_version() << ")\n";

  // ConfigureDomain / ConfigureLattice / ConfigureParameters
  const double Lx = cfg.real("domain_x"), Ly = cfg.real("domain_y");
  const double dX = cfg.real("lattice_dx"), dY = cfg.real("lattice_dy");
  const double xVol = cfg.real("lattice_xvol"), yVol = cfg.real("lattice_yvol");
  std::cout << "[Configuration] dX=" << dX << "\n[Configuration] dY=" << dY << "\n[Configuration] xVol=" << xVol
            << "\n[Configuration] yVol=" << yVol << "\n";
  if (!(dX > 0) || !(dY > 0) || !(Lx > 0) || !(Ly > 0)) {
    std::cerr << "[Error] domain_x, domain_y, lattice_dx and lattice_dy must be positive" << std::endl;
    return 1;
  }
  const long long ppx = (long long)std::ceil(xVol * Lx / dX) + 1;
  const long long ppy = (long long)std::ceil(yVol * Ly / dY) + 1;
  const long long N = ppx * ppy;
  std::cout << "[LatticeCreator] Total particles: " << N << std::endl;
  std::cout << "[LatticeCreator] Particles per direction: " << ppx << " " << ppy << " 1" << std::endl;
  std::vector<double> x(N), y(N), vx(N, 0.0), vy(N, 0.0);
  for (long long j = 0; j < ppy; ++j)
    for (long long i = 0; i < ppx; ++i) {
      x[i + ppx * j] = dX * i;
      y[i + ppx * j] = dY * j;
    }
  std::cout << "[Configuration] Lattice created in domain\n";

  const long long steps = cfg.integer("steps");
  const double dt = cfg.real("dt");
  const long long ckpt_freq = cfg.integer("checkpoint_write_frequency");
  const bool output_step0 = cfg.boolean("bool_output_first_step");
  const bool measure = cfg.boolean("bool_measure_neighborhood");
  const std::string order = cfg.str("order");
  const std::string ctype = cfg.str("compute_type");
  const std::string outdir = cfg.str("output_dir", ".");
  const long long header_freq = std::max(1LL, cfg.integer("header_frequency", 1));
  const long long snap_freq = cfg.integer("snapshot_write_frequency", 0);
  const std::string snap_prefix = cfg.str("snapshot_prefix", "snapshot_step_");
  if (output_step0) std::cout << "[Configuration] Printing step 0\n";
  if (measure) std::cout << "[Configuration] Cells neighborhood will be measured\n";
  if (ckpt_freq <= 0)
    std::cout << "[Configuration] checkpoint_write_frequency <= 0: no checkpoints are written\n";
  if (order != "morton" && order != "rowmajor") {
    std::cerr << "[Error] order must be morton or rowmajor, got '" << order << "'" << std::endl;
    return 1;
  }
  const bool lists = ctype == "lists" || ctype == "mp-lists";
  if (ctype != "gb300" && ctype != "sorted" && !lists) {
    std::cerr << "[Error] compute_type '" << ctype
              << "' is not served by this driver (gb300, sorted, lists or mp-lists)" << std::endl;
    return 1;
  }

  sphg_params p{};
  p.h = cfg.real("H", 1.0);
  p.dt = dt;
  p.k = cfg.real("GAS_CONSTANT", 30.0);
  p.rho0 = cfg.real("RHO_0", 25.0);
  p.mu = cfg.real("MU", 0.01);
  p.tol = 1e-12;
  p.gx = cfg.real("gravity_x", 0.0);
  p.gy = cfg.real("gravity_y", -10.0);
  p.mass = cfg.real("mass", 1.0);
  p.alpha = cfg.real("alpha", 0.0);
  p.c0 = cfg.real("c0", 0.0);
  p.lo[0] = 0.0;
  p.lo[1] = 0.0;
  p.hi[0] = Lx;
  p.hi[1] = Ly;
  p.order = order == "morton" ? SPHG_ORDER_MORTON : SPHG_ORDER_ROWMAJOR;
  p.periodic = (int32_t)cfg.integer("periodic", 0);
  sphg_options o;
  sphg_default_options(&o);
  o.precision = cfg.str("precision", "plain") == "split" ? SPHG_PRECISION_SPLIT : SPHG_PRECISION_PLAIN;
  o.use_graph = (int32_t)cfg.integer("use_graph", 1);
  o.compute = lists ? SPHG_COMPUTE_LISTS : SPHG_COMPUTE_SORTED;

  std::cout << "[Configuration] Domain size: " << Lx << " " << Ly << " 0\n";
  std::cout << "[Configuration] Particles=" << N << "\n[Configuration] steps=" << steps
            << "\n[Configuration] dt=" << dt << "\n[Configuration] output frequency=" << ckpt_freq << "\n";
  std::cout << "[Configuration] H=" << p.h << " GAS_CONSTANT=" << p.k << " RHO_0=" << p.rho0 << " MU=" << p.mu
            << "\n";
  std::cout << "[Configuration] Using " << order << " ordering, compute type gb300/"
            << (lists ? "lists" : "sorted") << " ("
            << (o.precision == SPHG_PRECISION_SPLIT ? "split" : "plain") << " precision)\n";
  std::cout << "[Configuration] Configuration complete." << std::endl;
  if (dry) return 0;

  sphg_sim* sim = nullptr;
  sphg_status st = sphg_create(&p, &o, N, &sim);
  if (st != SPHG_OK) die("sphg_create", st);

  // cells per direction of the reference's grid, for cells_<i>.txt
  const int gnx0 = (int)std::ceil(Lx / p.h), gny0 = (int)std::ceil(Ly / p.h);
  const int gnx = order == "morton" ? next_pow2(gnx0) : gnx0;
  const int gny = order == "morton" ? next_pow2(gny0) : gny0;
  const long long ncells = (long long)gnx * gny;
  std::vector<int32_t> keys;
  struct {
    long long num_cells = 0, num_empty = 0, avg_ppc = 0, min_ppc = 10000000, max_ppc = 0;
  } cell_stats;
  auto write_cells = [&](long long step) {
    keys.resize(N);
    sphg_status s2 = sphg_get_debug(sim, SPHG_DBG_KEYS, keys.data(), nullptr);
    if (s2 != SPHG_OK) die("sphg_get_debug", s2);
    std::vector<long long> cs(ncells, -1), ce(ncells, -1);
    for (long long i = 0; i < N; ++i) {
      const long long c = keys[i];
      if (c < 0 || c >= ncells) continue;
      if (i == 0 || keys[i - 1] != keys[i]) cs[c] = i;
      if (i == N - 1 || keys[i + 1] != keys[i]) ce[c] = i + 1;
    }
    std::ofstream f(outdir + "/cells_" + std::to_string(step) + ".txt");
    for (long long c = 0; c < ncells; ++c) f << "cell:" << c << "[" << cs[c] << "," << ce[c] << ")\n";
    // cell statistics of AvgNeighborsPerParticle::MeasureCells
    // (core/algorithmic/MeasureAverageNeighborsPerParticle.h:94-116)
    long long sum = 0;
    cell_stats.num_empty = 0;
    cell_stats.min_ppc = 10000000;
    cell_stats.max_ppc = 0;
    for (long long c = 0; c < ncells; ++c) {
      const long long k = ce[c] - cs[c];
      sum += k;
      cell_stats.max_ppc = std::max(cell_stats.max_ppc, k);
      if (k > 0) cell_stats.min_ppc = std::min(cell_stats.min_ppc, k);
      if (k == 0) ++cell_stats.num_empty;
    }
    cell_stats.num_cells = ncells;
    cell_stats.avg_ppc = ncells ? sum / ncells : 0;
  };
  std::vector<int64_t> offs;
  std::vector<int32_t> idx;
  auto assemble_lists = [&]() {
    timers.start("neighbor_list");
    int64_t total = 0;
    offs.resize(N + 1);
    sphg_status s2 = sphg_neighbor_lists(sim, offs.data(), nullptr, &total, nullptr);
    if (s2 == SPHG_OK) {
      idx.resize(total);
      s2 = sphg_neighbor_lists(sim, offs.data(), idx.data(), &total, nullptr);
    }
    if (s2 != SPHG_OK) die("sphg_neighbor_lists", s2);
    timers.stop("neighbor_list");
  };
  CheckpointWriter writer(outdir + "/positions_step_", (size_t)N);
  auto checkpoint = [&](long long step) {
    CheckpointWriter::Buf* b = writer.acquire();
    b->step = step;
    timers.start("cuda_buffer_copy");
    sphg_status s2 = sphg_download(sim, b->x.data(), b->y.data(), nullptr, nullptr, nullptr, nullptr, nullptr,
                                   nullptr, nullptr);
    timers.stop("cuda_buffer_copy");
    if (s2 != SPHG_OK) die("sphg_download", s2);
    writer.submit(b);
  };
  double diag[6];
  auto header = [&](long long step) {
    timers.start("IO");
    sphg_status s2 = sphg_diagnostics(sim, diag, nullptr);
    if (s2 != SPHG_OK) die("sphg_diagnostics", s2);
    std::cout << "Step= " << step << "\t N=" << (long long)diag[2] << "\t E_k=" << diag[0]
              << "\t |v|_max=" << diag[1] << std::endl;
    timers.stop("IO");
  };
  auto snapshot = [&](long long step) {
    uint64_t bytes = 0;
    sphg_status s2 = sphg_snapshot(sim, nullptr, &bytes, nullptr);
    std::vector<char> blob(bytes);
    if (s2 == SPHG_OK) s2 = sphg_snapshot(sim, blob.data(), &bytes, nullptr);
    if (s2 != SPHG_OK) die("sphg_snapshot", s2);
    std::ofstream f(outdir + "/" + snap_prefix + std::to_string(step) + ".bin", std::ios::binary);
    const int64_t s64 = step;
    f.write("SPHGRUN1", 8);
    f.write(reinterpret_cast<const char*>(&s64), 8);
    f.write(blob.data(), (std::streamsize)bytes);
  };

  long long first = 1;
  if (cfg.has("resume_from")) {
    std::ifstream f(cfg.str("resume_from"), std::ios::binary);
    std::vector<char> all((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    if (all.size() < 16 || std::memcmp(all.data(), "SPHGRUN1", 8) != 0) {
      std::cerr << "[Error] resume_from is not a snapshot written by this driver" << std::endl;
      return 1;
    }
    int64_t s64;
    std::memcpy(&s64, all.data() + 8, 8);
    st = sphg_restore(sim, all.data() + 16, all.size() - 16, nullptr);
    if (st != SPHG_OK) die("sphg_restore", st);
    st = sphg_preloop(sim, nullptr);
    if (st != SPHG_OK) die("sphg_preloop", st);
    first = s64 + 1;
    std::cout << "[Simulation] Resumed after step " << s64 << "\n";
  } else {
    // PreLoopComputation
    timers.start("cuda_buffer_copy");
    st = sphg_upload(sim, x.data(), y.data(), vx.data(), vy.data(), nullptr);
    timers.stop("cuda_buffer_copy");
    if (st != SPHG_OK) die("sphg_upload", st);
    timers.start("gpu_step");
    st = sphg_preloop(sim, nullptr);
    timers.stop("gpu_step");
    if (st != SPHG_OK) die("sphg_preloop", st);
    if (measure) {
      write_cells(0);
      assemble_lists();
    }
    std::cout << "[Simulation] Output step 0 positions\n";
    if (output_step0) checkpoint(0);
    header(0);
    if (snap_freq > 0 && steps > 0) snapshot(0);
  }

  // MainLoopComputation.  With a header after every iteration and no per-step
  // measurement, the iterations up to the next checkpoint or snapshot run as
  // one sphg_step_headers call (at most kBlock at a time) and their headers
  // are printed from its array: the same lines in the same order, without a
  // host synchronisation per iteration.
  constexpr long long kBlock = 256;
  std::vector<double> hbuf(6 * kBlock);
  auto next_multiple = [](long long i, long long f) { return (i + f - 1) / f * f; };
  timers.start("main_loop");
  for (long long i = first; i < steps;) {
    long long j = i;  // last iteration of this round
    if (!measure && header_freq == 1) {
      j = std::min(steps - 1, i + kBlock - 1);
      if (ckpt_freq > 0) j = std::min(j, next_multiple(i, ckpt_freq));
      if (snap_freq > 0) j = std::min(j, next_multiple(i, snap_freq));
      timers.start("gpu_step");
      st = sphg_step_headers(sim, j - i + 1, hbuf.data(), nullptr);
      if (st == SPHG_OK) st = sphg_stream_synchronize(nullptr);
      timers.stop("gpu_step");
      if (st != SPHG_OK) die("sphg_step_headers", st);
      timers.start("IO");
      for (long long k = i; k < j; ++k) {
        const double* h = hbuf.data() + 6 * (k - i);
        std::cout << "Step= " << k << "\t N=" << (long long)h[2] << "\t E_k=" << h[0] << "\t |v|_max=" << h[1]
                  << std::endl;
      }
      timers.stop("IO");
      if (ckpt_freq > 0 && j % ckpt_freq == 0) {
        timers.start("IO");
        checkpoint(j);
        timers.stop("IO");
      }
      header(j);  // also reads the kernels' error words
      if (snap_freq > 0 && j % snap_freq == 0) snapshot(j);
      i = j + 1;
      continue;
    }
    timers.start("gpu_step");
    st = sphg_step(sim, 1, nullptr);
    timers.stop("gpu_step");
    if (st != SPHG_OK) die("sphg_step", st);
    if (measure) {
      write_cells(i);
      assemble_lists();
    }
    if (ckpt_freq > 0 && i % ckpt_freq == 0) {
      timers.start("IO");
      checkpoint(i);
      timers.stop("IO");
    }
    if (i % header_freq == 0 || i == steps - 1) header(i);
    if (snap_freq > 0 && i % snap_freq == 0) snapshot(i);
    ++i;
  }
  writer.finish();
  timers.stop("main_loop");
  sphg_destroy(sim);
  timers.print();
  timers.append_file(outdir + "/timer_manager.data", steps, N);
  if (measure && !offs.empty()) {
    // AvgNeighborsPerParticle::Measure + PrintToFile on the last iteration's lists
    // (core/algorithmic/MeasureAverageNeighborsPerParticle.h:66-92,118-134): neighbours
    // per particle (self included), integer average, population standard deviation
    long long sum = 0, mn = N, mx = 0;
    for (long long i = 0; i < N; ++i) {
      const long long k = offs[i + 1] - offs[i];
      sum += k;
      mn = std::min(mn, k);
      mx = std::max(mx, k);
    }
    const long long avg = N ? sum / N : 0;
    double dev = 0.0;
    for (long long i = 0; i < N; ++i) {
      const double k = (double)(offs[i + 1] - offs[i]) - (double)avg;
      dev += k * k;
    }
    dev = N ? std::sqrt(dev / (double)N) : 0.0;
    const std::string name = outdir + "/neighborhood_and_cells.data";
    const bool fresh = !std::ifstream(name).good();
    std::ofstream f(name, std::ios::app);
    if (fresh) {
      for (const char* c : {"avg_npp", "min_npp", "max_npp", "stddev_npp", "#cells", "#empty_cells", "avg_ppc",
                            "min_ppc"})
        f << std::fixed << std::setw(20) << std::left << c << "\t";
      f << std::fixed << std::setw(20) << std::left << "max_ppc" << "\n";
    }
    f << std::fixed << std::setw(20) << std::left << avg << "\t" << std::setw(20) << mn << "\t" << std::setw(20) << mx
      << "\t" << std::setw(20) << dev << "\t" << std::setw(20) << cell_stats.num_cells << "\t" << std::setw(20)
      << cell_stats.num_empty << "\t" << std::setw(20) << cell_stats.avg_ppc << "\t" << std::setw(20)
      << cell_stats.min_ppc << "\t" << std::setw(20) << cell_stats.max_ppc << "\n";
  }
  if (writer.failed()) {
    std::cerr << "[Error] a checkpoint file could not be written" << std::endl;
    return 1;
  }
  return 0;
}

// Headless solver: the reference's command-line solver (src/solver.cpp) over the GB300 step.
//
// Same flags and defaults as the reference (src/solver.cpp:25-41, 151-218): --steps, --cubes,
// --cube-res, --dim, --E, --nu, --gravity, --material-model, --cube<n>-x / --cube<n>-y (the
// min and max of cube n's lattice on every axis, as generate_cubes reads them), --dump,
// --help.  The 3D path, empty in the reference (src/solver.cpp:211-216), runs here.
//
// Differences, all additions:
//   * the cubes are built on the device (nclr_cubes_device) and the simulation is created from
//     device arrays (nclr_create_device);
//   * --dump writes one binary file, <out>/dump.nclr, instead of the per-step text files of
//     src/solver.cpp:75-131: the state before every advance() (as solve_mpm collects it) and
//     the grid of the previous advance() (zeros at step 0), copied device -> host on a copy
//     stream through a ring of pinned buffers and written by a writer thread while the next
//     steps run.  nuclearmpm_gb300.dumpio reads it into the structure python/ioutils.py
//     builds from the text files;
//   * --render writes every --render-every'th step as a PPM frame drawn on the device
//     (nclr_render_device: the canvas of src/solver.cpp:184-201, headless);
//   * --out DIR (default tmp), --res (default 64, the reference's kGridResolution),
//     --physics reference|corrected, --stress corotated|neohookean, --device N.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <filesystem>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "nclr_gpu.h"

namespace fs = std::filesystem;

namespace {

constexpr uint32_t kColor = 0xED553B;  // src/solver.cpp:18
constexpr float kDt = 1e-4f;           // src/solver.cpp:24
constexpr int kWindowSize = 800;       // src/solver.cpp:15

void help_msg() {
  std::printf(
      "Usage: ./nclr_solver [OPTIONS]\n"
      "\tNuclearMPM headless solver (GB300)\n"
      "Options:\n"
      "\t--steps\tINTEGER\t[default:1000]\tThe number of simulation steps\n"
      "\t--cubes\tINTEGER\t[default:1]\tThe number of cubes to add\n"
      "\t--cube-res\tINTEGER\t[default:25]\tThe resolution of each cube\n"
      "\t--dim\tINTEGER\t[default:2]\tThe number of dimensions to run the sim in [2d or 3d]\n"
      "\t--E\tFLOAT\t[default:1000.0]\tThe young's modulus of the shape(s)\n"
      "\t--nu\tFLOAT\t[default:0.3]\tThe poisson's ratio of the shape(s)\n"
      "\t--gravity\tFLOAT\t[default:-100.0]\tThe gravitational forces\n"
      "\t--material-model\t[jelly, snow, liquid]\t[default:jelly]\tThe material model to use\n"
      "\t--cube[n]-[xy]\t\tCube n's lattice min (x) and max (y) on every axis (0.1-0.9)\n"
      "\t--dump\tDump particle and grid state at each timestep into <out>/dump.nclr\n"
      "\t--render\tWrite PPM frames into <out>/frames\n"
      "\t--render-every\tINTEGER\t[default:10]\tSteps between frames\n"
      "\t--out\tDIR\t[default:tmp]\tOutput directory\n"
      "\t--res\tINTEGER\t[default:64]\tGrid resolution\n"
      "\t--physics\t[reference, corrected]\t[default:reference]\n"
      "\t--stress\t[corotated, neohookean]\t[default:corotated]\tThe stress model\n"
      "\t--device\tINTEGER\t[default:0]\tCUDA device\n"
      "\t--help\tShow this message and exit\n");
}

// `--key value`, `--key=value` and bare `--key` (true), as the reference's flags library reads
// them.
struct Args {
  std::map<std::string, std::string> kv;
  Args(int argc, char **argv) {
    for (int i = 1; i < argc; ++i) {
      std::string a = argv[i];
      if (a.rfind("--", 0) != 0) continue;
      a = a.substr(2);
      const size_t eq = a.find('=');
      if (eq != std::string::npos) {
        kv[a.substr(0, eq)] = a.substr(eq + 1);
      } else if (i + 1 < argc && std::string(argv[i + 1]).rfind("--", 0) != 0) {
        kv[a] = argv[++i];
      } else {
        kv[a] = "true";
      }
    }
  }
  bool has(const std::string &k) const { return kv.count(k) != 0; }
  std::string str(const std::string &k, const std::string &d) const {
    auto it = kv.find(k);
    return it == kv.end() ? d : it->second;
  }
  double num(const std::string &k, double d) const {
    auto it = kv.find(k);
    return it == kv.end() ? d : std::atof(it->second.c_str());
  }
  bool flag(const std::string &k) const {
    auto it = kv.find(k);
    return it != kv.end() && it->second != "false" && it->second != "0";
  }
};

#define CK(call)                                                                       \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      std::fprintf(stderr, "%s: %s\n", #call, cudaGetErrorString(e_));                 \
      std::exit(EXIT_FAILURE);                                                         \
    }                                                                                  \
  } while (0)

void check(nclr_status st, nclr_sim *sim, const char *what) {
  if (st == NCLR_OK) return;
  std::fprintf(stderr, "%s failed (%d): %s\n", what, (int)st, nclr_last_error(sim));
  std::exit(st == NCLR_ERR_OUT_OF_RANGE ? 3 : EXIT_FAILURE);
}

// dump.nclr: this header, then one record per dumped step.  Little-endian, no padding.
#pragma pack(push, 1)
struct DumpHeader {
  char magic[8];  // "NCLRDMP1"
  uint32_t dim, res, model, physics;
  int64_t n;
  float dt, mu0, lambda0, hardening;
};
// record: int64 step, float timestep, float reserved, then x (n*dim), v (n*dim), F (n*dim*dim),
// C (n*dim*dim), Jp (n), grid velocity ((res+1)^dim * dim), grid mass ((res+1)^dim) as float32
#pragma pack(pop)

// The asynchronous dump: a ring of device and pinned host slots, a copy stream, a writer thread.
class Dumper {
 public:
  Dumper(const std::string &path, const DumpHeader &h, nclr_sim *sim, int slots = 3)
      : sim_(sim), dim_(h.dim), n_(h.n), nodes_(1) {
    for (uint32_t d = 0; d < h.dim; ++d) nodes_ *= (int64_t)h.res + 1;
    floats_ = n_ * (2 * dim_ + 2 * dim_ * dim_ + 1) + nodes_ * (dim_ + 1);
    f_ = std::fopen(path.c_str(), "wb");
    if (!f_) {
      std::fprintf(stderr, "cannot open %s\n", path.c_str());
      std::exit(EXIT_FAILURE);
    }
    std::fwrite(&h, sizeof(h), 1, f_);
    CK(cudaStreamCreateWithFlags(&copy_, cudaStreamNonBlocking));
    slots_.resize((size_t)slots);
    for (auto &s : slots_) {
      CK(cudaMalloc((void **)&s.dev, sizeof(float) * (size_t)floats_));
      CK(cudaMallocHost((void **)&s.host, sizeof(float) * (size_t)floats_));
      CK(cudaEventCreateWithFlags(&s.ready, cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&s.copied, cudaEventDisableTiming));
    }
    writer_ = std::thread([this] { write_loop(); });
  }

  // Enqueues the state before step `step` (and the grid of the previous step) on the
  // simulation's stream, its download on the copy stream, and its writing on the thread.
  void dump(int64_t step) {
    const size_t k = (size_t)(step % (int64_t)slots_.size());
    Slot &s = slots_[k];
    {
      std::unique_lock<std::mutex> lk(mu_);
      cv_.wait(lk, [&] { return !s.busy; });
      s.busy = true;
    }
    cudaStream_t st = static_cast<cudaStream_t>(nclr_stream(sim_));
    float *x = s.dev, *v = x + n_ * dim_, *F = v + n_ * dim_, *C = F + n_ * dim_ * dim_;
    float *Jp = C + n_ * dim_ * dim_, *gv = Jp + n_, *gm = gv + nodes_ * dim_;
    check(nclr_get_particles_device(sim_, x, v, F, C, Jp), sim_, "particles()");
    if (step > 0) {
      check(nclr_get_grid_device(sim_, gv, gm), sim_, "grid()");
    } else {  // solve_mpm dumps an empty grid before the first step (src/solver.cpp:51-55)
      CK(cudaMemsetAsync(gv, 0, sizeof(float) * (size_t)(nodes_ * (dim_ + 1)), st));
    }
    CK(cudaEventRecord(s.ready, st));
    CK(cudaStreamWaitEvent(copy_, s.ready, 0));
    CK(cudaMemcpyAsync(s.host, s.dev, sizeof(float) * (size_t)floats_, cudaMemcpyDeviceToHost, copy_));
    CK(cudaEventRecord(s.copied, copy_));
    {
      std::lock_guard<std::mutex> lk(mu_);
      queue_.push_back({k, step});
    }
    cv_.notify_all();
  }

  ~Dumper() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      done_ = true;
    }
    cv_.notify_all();
    writer_.join();
    std::fclose(f_);
    for (auto &s : slots_) {
      cudaFree(s.dev);
      cudaFreeHost(s.host);
      cudaEventDestroy(s.ready);
      cudaEventDestroy(s.copied);
    }
    cudaStreamDestroy(copy_);
  }

  int64_t bytes_written() const { return written_; }

 private:
  struct Slot {
    float *dev = nullptr, *host = nullptr;
    cudaEvent_t ready = nullptr, copied = nullptr;
    bool busy = false;
  };

  void write_loop() {
    for (;;) {
      std::pair<size_t, int64_t> job;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return done_ || !queue_.empty(); });
        if (queue_.empty()) return;
        job = queue_.front();
        queue_.pop_front();
      }
      Slot &s = slots_[job.first];
      CK(cudaEventSynchronize(s.copied));
      const int64_t step = job.second;
      // the reference's timestep column: kDt * step, and kDt at step 0 (src/solver.cpp:91)
      const float ts[2] = {step > 0 ? kDt * (float)step : kDt, 0.0f};
      std::fwrite(&step, sizeof(step), 1, f_);
      std::fwrite(ts, sizeof(ts), 1, f_);
      std::fwrite(s.host, sizeof(float), (size_t)floats_, f_);
      written_ += (int64_t)(sizeof(step) + sizeof(ts) + sizeof(float) * (size_t)floats_);
      {
        std::lock_guard<std::mutex> lk(mu_);
        s.busy = false;
      }
      cv_.notify_all();
    }
  }

  nclr_sim *sim_;
  int64_t dim_, n_, nodes_, floats_;
  FILE *f_ = nullptr;
  cudaStream_t copy_ = nullptr;
  std::vector<Slot> slots_;
  std::deque<std::pair<size_t, int64_t>> queue_;
  std::mutex mu_;
  std::condition_variable cv_;
  bool done_ = false;
  int64_t written_ = 0;
  std::thread writer_;
};

void write_ppm(const std::string &path, const std::vector<uint32_t> &rgb, int w, int h) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) return;
  std::fprintf(f, "P6\n%d %d\n255\n", w, h);
  std::vector<unsigned char> row((size_t)w * 3);
  for (int j = 0; j < h; ++j) {
    for (int i = 0; i < w; ++i) {
      const uint32_t c = rgb[(size_t)j * w + i];
      row[(size_t)i * 3] = (unsigned char)(c >> 16);
      row[(size_t)i * 3 + 1] = (unsigned char)(c >> 8);
      row[(size_t)i * 3 + 2] = (unsigned char)c;
    }
    std::fwrite(row.data(), 1, row.size(), f);
  }
  std::fclose(f);
}

}  // namespace

int main(int argc, char **argv) {
  const Args args(argc, argv);
  const bool help = args.flag("help");
  const std::string material = args.str("material-model", "jelly");
  if (material != "jelly" && material != "snow" && material != "liquid") {
    std::fprintf(stderr, "Invalid Option: %s\n", material.c_str());
    help_msg();
    return EXIT_FAILURE;
  }
  if (help || argc == 1) help_msg();
  if (help) return EXIT_SUCCESS;

  const int64_t steps = (int64_t)args.num("steps", 1000);
  const int cubes = (int)args.num("cubes", 1);
  const int cube_res = (int)args.num("cube-res", 25);
  const int dim = (int)args.num("dim", 2);
  const float E = (float)args.num("E", 1000.0), nu = (float)args.num("nu", 0.3);
  const float gravity = (float)args.num("gravity", -100.0);
  const int res = (int)args.num("res", 64);
  const bool dump = args.flag("dump"), render = args.flag("render");
  const int render_every = std::max(1, (int)args.num("render-every", 10));
  const fs::path out = args.str("out", "tmp");
  const int device = (int)args.num("device", 0);
  const std::string physics = args.str("physics", "reference");
  const std::string stress = args.str("stress", "corotated");
  if (stress != "corotated" && stress != "neohookean") {
    std::fprintf(stderr, "Invalid Option: %s\n", stress.c_str());
    return EXIT_FAILURE;
  }
  if (dim != 2 && dim != 3) {
    std::fprintf(stderr, "--dim must be 2 or 3\n");
    return EXIT_FAILURE;
  }
  const int model = material == "snow" ? NCLR_SNOW : material == "liquid" ? NCLR_LIQUID : NCLR_JELLY;

  // generate_cubes (src/solver.cpp:133-149): every cube needs --cube<n>-x and --cube<n>-y
  std::vector<float> lo, hi;
  for (int c = 0; c < cubes; ++c) {
    const std::string kx = "cube" + std::to_string(c) + "-x", ky = "cube" + std::to_string(c) + "-y";
    if (!args.has(kx) || !args.has(ky)) {
      std::fprintf(stderr, "Cube: %d is missing coordinates\n", c);
      return EXIT_FAILURE;
    }
    lo.push_back((float)args.num(kx, 0.0));
    hi.push_back((float)args.num(ky, 0.0));
  }
  int64_t per = cube_res;
  for (int d = 1; d < dim; ++d) per *= cube_res;
  const int64_t n = per * cubes;

  CK(cudaSetDevice(device));
  float *x = nullptr;
  CK(cudaMalloc((void **)&x, sizeof(float) * (size_t)std::max<int64_t>(n * dim, 1)));
  check(nclr_cubes_device(dim, cubes, cube_res, lo.data(), hi.data(), x, nullptr), nullptr,
        "cube construction");
  nclr_options opt;
  nclr_default_options(&opt);
  opt.device = device;
  opt.physics = physics == "corrected" ? NCLR_PHYSICS_CORRECTED : NCLR_PHYSICS_REFERENCE;
  opt.stress_model = stress == "neohookean" ? NCLR_STRESS_NEOHOOKEAN : NCLR_STRESS_COROTATED;
  nclr_sim *sim = nullptr;
  check(nclr_create_device(&sim, dim, n, x, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                           nullptr, model, res, kDt, E, nu, gravity, &opt),
        nullptr, "simulation");
  CK(cudaFree(x));

  std::printf("Running simulation: %lld particles, %dD, %s, %lld steps\n", (long long)n, dim,
              material.c_str(), (long long)steps);
  std::unique_ptr<Dumper> dumper;
  if (dump) {
    fs::create_directories(out);
    DumpHeader h{};
    std::memcpy(h.magic, "NCLRDMP1", 8);
    h.dim = (uint32_t)dim;
    h.res = (uint32_t)res;
    h.model = (uint32_t)model;
    h.physics = (uint32_t)opt.physics;
    h.n = n;
    h.dt = kDt;
    check(nclr_get_lame(sim, &h.mu0, &h.lambda0), sim, "lame");
    h.hardening = model == NCLR_SNOW ? 10.0f : model == NCLR_JELLY ? 0.3f : 1.0f;  // kXHardening
    dumper.reset(new Dumper((out / "dump.nclr").string(), h, sim));
  }
  float *rx = nullptr;
  uint32_t *rgba_d = nullptr;
  std::vector<uint32_t> rgba;
  if (render) {
    fs::create_directories(out / "frames");
    CK(cudaMalloc((void **)&rx, sizeof(float) * (size_t)std::max<int64_t>(n * dim, 1)));
    CK(cudaMalloc((void **)&rgba_d, sizeof(uint32_t) * kWindowSize * kWindowSize));
    rgba.resize((size_t)kWindowSize * kWindowSize);
  }

  const auto t0 = std::chrono::steady_clock::now();
  if (!dump && !render) {
    check(nclr_advance(sim, steps), sim, "advance()");  // one call: CUDA graphs over the steps
  } else {
    cudaStream_t st = static_cast<cudaStream_t>(nclr_stream(sim));
    for (int64_t step = 0; step < steps; ++step) {
      if (dumper) dumper->dump(step);
      if (render && step % render_every == 0) {
        check(nclr_get_particles_device(sim, rx, nullptr, nullptr, nullptr, nullptr), sim, "particles()");
        check(nclr_render_device(rx, n, dim, nullptr, kColor, kWindowSize, kWindowSize, 2.0f, rgba_d, st),
              sim, "render");
        CK(cudaMemcpyAsync(rgba.data(), rgba_d, sizeof(uint32_t) * rgba.size(), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        char name[32];
        std::snprintf(name, sizeof(name), "%06lld.ppm", (long long)step);
        write_ppm((out / "frames" / name).string(), rgba, kWindowSize, kWindowSize);
      }
      check(nclr_advance(sim, 1), sim, "advance()");
    }
  }
  CK(cudaDeviceSynchronize());
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  int64_t written = 0;
  if (dumper) {
    dumper.reset();  // drains the writer
    written = (int64_t)fs::file_size(out / "dump.nclr");
  }
  std::printf("Simulation done: %.3f s, %.3e particle-steps/s%s\n", secs,
              secs > 0 ? (double)n * (double)steps / secs : 0.0,
              dump ? (", dump " + std::to_string(written) + " bytes").c_str() : "");
  if (rx) cudaFree(rx);
  if (rgba_d) cudaFree(rgba_d);
  nclr_destroy(sim);
  return EXIT_SUCCESS;
}

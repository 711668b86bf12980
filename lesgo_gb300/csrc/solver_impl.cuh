// Host orchestration of the GB300 LES step: one Solver<R, A> per handle owns
// the device field store, the FFT tables, the scratch spectra, one CUDA
// stream and the captured CUDA graphs of the steady steps.  Each precision
// form instantiates the template in a translation unit of its own
// (solver_fp32.cu, solver_fp64.cu, solver_dw.cu, compiled in parallel); the
// C ABI (solver.cu) reaches them through make_solver_*.
#pragma once
#include "lesgo_gpu.h"
#include "kernels.cuh"
#include "convec_rows.cuh"
#include "tc_dft.cuh"
#include "restart_io.hpp"
#include "conf.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <complex>
#include <cstring>
#include <array>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace lesgo {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CK(x)                                                                                 \
  do {                                                                                        \
    cudaError_t e_ = (x);                                                                     \
    if (e_ != cudaSuccess)                                                                    \
      throw Error(e_ == cudaErrorMemoryAllocation ? LESGO_ERR_NOMEM : LESGO_ERR_CUDA,         \
                  std::string(#x) + ": " + cudaGetErrorString(e_));                           \
  } while (0)

static const long double kPiL = 3.141592653589793238462643383279502884L;
static const double kPi = 3.1415926535897932384626433;   // param.f90:94

// Radix schedule for a 2^a 3^b length: radix-8 stages, then 4s, at most one
// 2, then 3s.  max8 = false (the double-word transforms, whose butterflies
// are compiled for radix 4, 3 and 2 only): 4s, at most one 2, then 3s.
static std::vector<int> factorize(int n, bool max8 = true) {
  int m = n, e2 = 0, e3 = 0;
  while (m % 2 == 0) { m /= 2; ++e2; }
  while (m % 3 == 0) { m /= 3; ++e3; }
  if (m != 1 || n < 1) throw Error(LESGO_ERR_UNSUPPORTED, "transform length " + std::to_string(n) + " is not 2^a 3^b");
  std::vector<int> r;
  if (!max8) {
    for (int i = 0; i < e2 / 2; ++i) r.push_back(4);
    if (e2 % 2) r.push_back(2);
  } else if (e2 % 3 == 0) { for (int i = 0; i < e2 / 3; ++i) r.push_back(8); }
  else if (e2 % 3 == 1) {
    if (e2 >= 4) { for (int i = 0; i < (e2 - 4) / 3; ++i) r.push_back(8); r.push_back(4); r.push_back(4); }
    else r.push_back(2);
  } else { for (int i = 0; i < (e2 - 2) / 3; ++i) r.push_back(8); r.push_back(4); }
  for (int i = 0; i < e3; ++i) r.push_back(3);
  if ((int)r.size() > kMaxStages) throw Error(LESGO_ERR_UNSUPPORTED, "too many radix stages");
  return r;
}

// ---------------------------------------------------------------------------
// Derived run parameters (input_util.f90:196-235, 403-409, 534-542; sgs_param.f90:187)
// ---------------------------------------------------------------------------
struct Derived {
  lesgo_params_t p;
  int nx, ny, nz, nz_tot, ld, lh, nx2, ny2, ld_big, K;
  double dx, dy, dz, tadv1, tadv2, mpfx, mpfy, delta, nu, lagran_dt;
  std::vector<lesgo_turbine_t> turbines;

  explicit Derived(const lesgo_params_t& in) : p(in) {
    if (p.nx < 4 || p.ny < 2 || p.nz_tot < 3) throw Error(LESGO_ERR_ARG, "grid too small");
    if (p.nx % 4 != 0 || p.ny % 2 != 0) throw Error(LESGO_ERR_UNSUPPORTED, "nx must be a multiple of 4 and ny even");
    if (p.sgs_model != 5) throw Error(LESGO_ERR_UNSUPPORTED, "only sgs_model = 5 (Lagrangian scale-dependent)");
    if (p.ifilter != 1) throw Error(LESGO_ERR_UNSUPPORTED, "only ifilter = 1 (spectral cut-off)");
    if (p.lbc_mom < 0 || p.lbc_mom > 2 || p.ubc_mom < 0 || p.ubc_mom > 2)
      throw Error(LESGO_ERR_UNSUPPORTED, "lbc_mom / ubc_mom must be 0, 1 or 2");
    if (p.cs_count < 1) throw Error(LESGO_ERR_ARG, "cs_count must be >= 1");
    if (p.precision != LESGO_FP64 && p.precision != LESGO_MIXED && p.precision != LESGO_FP64_DW)
      throw Error(LESGO_ERR_ARG, "precision");
    if (p.dt <= 0 || p.L_x <= 0 || p.L_y <= 0 || p.L_z <= 0 || p.zo <= 0) throw Error(LESGO_ERR_ARG, "non-positive length/time");
    if (p.use_cfl_dt && !(p.cfl > 0)) throw Error(LESGO_ERR_ARG, "use_cfl_dt needs cfl > 0");
    nx = p.nx; ny = p.ny;
    const int nproc = 1;
    nz = p.nz_tot / nproc + 1;
    nz_tot = (nz - 1) * nproc + 1;
    nx2 = 3 * nx / 2; ny2 = 3 * ny / 2;
    lh = nx / 2 + 1; ld = 2 * lh;
    ld_big = 2 * (nx2 / 2 + 1);
    K = nx / 2;
    dx = p.L_x / nx;
    dy = p.L_y / ny;
    dz = p.L_z / (nz_tot - 1);
    tadv1 = 1.5; tadv2 = 1.0 - tadv1;
    mpfx = p.mean_p_force_x; mpfy = p.mean_p_force_y;
    if (p.use_mean_p_force && p.eval_mean_p_force) {
      mpfx = mpfx / std::sqrt(mpfx * mpfx + mpfy * mpfy) / p.L_z;
      mpfy = mpfy / std::sqrt(mpfx * mpfx + mpfy * mpfy) / p.L_z;
    }
    delta = 1.0 * std::pow(dx * dy * dz, 1.0 / 3.0);
    nu = p.molec ? p.nu_molec / (p.u_star * p.z_i) : 0.0;
    lagran_dt = (double)p.cs_count * p.dt;
    if (p.n_turbines > 0) {
      if (!p.turbines) throw Error(LESGO_ERR_ARG, "turbines == NULL");
      turbines.assign(p.turbines, p.turbines + p.n_turbines);
    }
    this->p.turbines = nullptr;
  }
};

}  // namespace lesgo

#include "turbine_host.hpp"

namespace lesgo {

// ---------------------------------------------------------------------------
// Solver: `capacity` slots of one grid size, the first n_active of which hold
// live LES instances (stable ids map to slots; removal compacts).  Every
// kernel processes all active instances in one launch.  A single-instance
// handle is a batch of capacity one.
// ---------------------------------------------------------------------------
struct InstanceSpec {
  double zo;
  uint64_t seed;
  std::vector<lesgo_turbine_t> turbines;
  Schedules sched;   // control schedules, rows of (time, one value per turbine)
};

class SolverBase {
 public:
  virtual ~SolverBase() {}
  virtual const Derived& der() const = 0;
  virtual int capacity() const = 0;
  virtual int active() const = 0;
  virtual int add_instance(const InstanceSpec& spec) = 0;
  virtual void remove_instance(int id) = 0;
  // wait = false: stream-ordered, returns once the copy is queued
  virtual void set_field(int id, int f, const double* h, int lbz, int nzhi, bool wait = true) = 0;
  virtual void get_field(int id, int f, double* h, int lbz, int nzhi, bool wait = true) = 0;
  virtual void init_ic(int id, uint64_t seed) = 0;
  virtual void filt_da(int f, int dx, int dy) = 0;
  virtual void ddxy(int f, int dx, int dy) = 0;   // dx or dy may be -1
  virtual void ddz(int f, int dfdz, bool uv) = 0;
  virtual void test_filter(int f, int level) = 0;
  virtual void wallstress() = 0;
  virtual void sgs_stag() = 0;
  virtual void divstress(int which) = 0;
  virtual void convec() = 0;
  virtual void turbines_forcing() = 0;
  virtual void begin_step() = 0;
  virtual void rhs_assemble() = 0;
  virtual void ab2() = 0;
  virtual void press_stag_array() = 0;
  virtual void rhs_sub_dp() = 0;
  virtual void project() = 0;
  virtual void step(int n) = 0;
  virtual int sync() = 0;
  virtual void diag(int id, double* out4) = 0;
  virtual void counters(int id, int* jt, int* jt_total) const = 0;
  virtual void turbine_state(int id, double* udT, double* fn, double* pw, int n) = 0;
  virtual void turbine_schedule(int id, int which, int nt, const double* rows) = 0;
  virtual void turbine_controls(int id, double* th1, double* th2, double* ctp, int n) = 0;
  virtual int launches_per_step(int with_sgs) const = 0;
  virtual void profile(int enable) = 0;
  virtual std::string profile_report() = 0;
  virtual void* stream() const = 0;
  virtual int tridag(const double* a, const double* b, const double* c, const double* r, double* u, int lh, int ny,
                     int n) = 0;
  virtual void tavg_config(int nstart, int nend, int nskip) = 0;
  virtual void tavg_sample() = 0;
  virtual void tavg_get(int id, int which, double* host, int lbz, int nzhi) = 0;
  virtual void tavg_profile(int id, int which, double* prof, int n) = 0;
  virtual double tavg_total_time(int id) = 0;
  virtual void checkpoint_write(int id, const std::string& path, int mpi_names) = 0;
  virtual int checkpoint_read(int id, const std::string& path) = 0;
  virtual double sim_time(int id) = 0;
  virtual double time_step(int id) = 0;
  virtual void diag_log_config(int every, int capacity) = 0;
  virtual void autotune(int* xtarget, int* ybudget) = 0;
  virtual void diag_log_sample() = 0;
  virtual int diag_log_read(int id, double* out, int maxrows) = 0;
};

// Whether the convective term's 3/2-grid x-rows run as one pass
// (k_convec_rows: c2r, products and r2c in shared memory) or as three
// (xinv to six 3/2-grid fields in HBM, products, xfwd).  One pass for the
// mixed and the double-word forms, three for the FP64 form, whose FP64
// transforms leave the one-pass kernel slower (measured at 128^3: 8.06
// against 7.87 ms per step); LESGO_CONVEC_ROWS=1 / 0 chooses for every form.
static bool convec_rows_enabled(int precision) {
  const char* e = std::getenv("LESGO_CONVEC_ROWS");
  if (e) return std::strcmp(e, "0") != 0;
  return precision != LESGO_FP64;
}

// A kernel's dynamic shared-memory limit (cudaFuncAttributeMaxDynamicSharedMemorySize)
// belongs to the function, not to a launch, and a replayed CUDA graph
// launches its kernel nodes against the value current at replay.  Handles
// of different grids share the kernel instances, so a handle that set a
// smaller limit than another handle's captured node needs would break that
// node's replay.  The limit is therefore only ever raised, per device,
// under a lock (handles may live on several host threads).
static void raise_smem_limit(const void* kern, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> limit;
  int dev = 0;
  CK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  size_t& cur = limit[{dev, kern}];
  if (bytes <= cur) return;
  CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  cur = bytes;
}

// Device bytes of a handle (the admission footprint of a batch).
static long long footprint_bytes(const Derived& d, int cap) {
  const long long rs = d.p.precision == LESGO_MIXED ? 4 : 8;
  const long long plane = (long long)d.ld * d.ny, pbig = (long long)d.ld_big * d.ny2;
  const long long nf = (long long)(d.nz + 1) * plane;
  const long long vs = (long long)d.nz * d.ny * d.K, vb = (long long)d.nz * d.ny2 * d.K, ps = (long long)d.ny * d.K;
  long long b = 0;
  b += (LESGO_NFIELDS + 4 + (d.turbines.empty() ? 0 : 1)) * nf * rs;   // fields, interpolation temps, fza on uv
  b += 4 * plane * rs;                                                  // wall planes
  if (!convec_rows_enabled(d.p.precision)) b += 6 * (long long)(d.nz + 1) * pbig * rs;   // 3/2-grid fields
  b += (std::max({21 * vs, 6 * vs, 3 * vb}) + std::max({42 * vs, 6 * vb, 9 * vs}) + 4 * ps) * 2 * rs;   // spectra
  b += (std::max(6 * vs, 3 * vb) + std::max(6 * vb, 3 * vs)) * 2 * rs;                             // convec spectra
  b += (3 * vs + 2 * ps + (long long)(d.nz + 1) * ps) * 16;                                          // FP64 pressure
  return b * cap + 2LL * (d.nz + 2) * ps * 8;                                                       // Thomas pivots
}

// Host rounding of a table value to the transforms' arithmetic type (the
// double-word split keeps the rounded-off rest as the low part).
template <typename A> struct HostCvt;
template <> struct HostCvt<float> { static float from(long double v) { return (float)v; } };
template <> struct HostCvt<double> { static double from(long double v) { return (double)v; } };
template <> struct HostCvt<df64> {
  static df64 from(long double v) {
    const float h = (float)v;
    return df64{h, (float)(v - (long double)h)};
  }
};

// R: the fields' storage and pointwise arithmetic; A: the transforms'
// arithmetic and spectral storage (R itself, or df64 for FP64 fields).
template <typename R, typename A = R>
class Solver : public SolverBase {
  using T2 = cplx<A>;

 public:
  Solver(const Derived& d, int capacity) : d_(d), cap_(capacity) {
    if (capacity < 1) throw Error(LESGO_ERR_ARG, "capacity must be >= 1");
    CK(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
    const int nx = d_.nx, ny = d_.ny, nz = d_.nz;
    kp_.nx = nx; kp_.ny = ny; kp_.nz = nz; kp_.ld = d_.ld; kp_.lh = d_.lh;
    kp_.nx2 = d_.nx2; kp_.ny2 = d_.ny2; kp_.ld_big = d_.ld_big; kp_.K = d_.K;
    kp_.plane = (long long)d_.ld * ny;
    kp_.plane_big = (long long)d_.ld_big * d_.ny2;
    kp_.dx = d_.dx; kp_.dy = d_.dy; kp_.dz = d_.dz;
    kp_.L_x = d_.p.L_x; kp_.L_y = d_.p.L_y; kp_.L_z = d_.p.L_z;
    kp_.vonk = d_.p.vonk; kp_.zo = d_.p.zo; kp_.nu = d_.nu; kp_.delta = d_.delta;
    kp_.mpfx = d_.mpfx; kp_.mpfy = d_.mpfy;
    kp_.nu_nd = d_.p.nu_molec / (d_.p.z_i * d_.p.u_star);
    kp_.ubot = d_.p.ubot; kp_.utop = d_.p.utop;
    kp_.lbc = d_.p.lbc_mom; kp_.ubc = d_.p.ubc_mom; kp_.use_mpf = d_.p.use_mean_p_force;
    kp_.turbines = 0;
    kp_.ninst = 0;
    kp_.istride = (long long)(nz + 1) * kp_.plane;
    kp_.fnx = FastDiv((unsigned)nx); kp_.fny = FastDiv((unsigned)ny); kp_.fnz = FastDiv((unsigned)nz);
    kp_.idx = 1.0 / kp_.dx; kp_.idy = 1.0 / kp_.dy; kp_.idz = 1.0 / kp_.dz;
    kp_.iLx = 1.0 / kp_.L_x; kp_.iLy = 1.0 / kp_.L_y;
    if ((long long)nx * ny * (nz + 1) * capacity >= (1LL << 31))
      throw Error(LESGO_ERR_UNSUPPORTED, "more than 2^31 grid points in one handle");
    kp_.istride_big = (long long)(nz + 1) * kp_.plane_big;
    nfield_ = kp_.istride * cap_;
    for (int f = 0; f < LESGO_NFIELDS; ++f) F_[f] = alloc<R>(nfield_);
    for (int f = 0; f < 4; ++f) Ftmp_[f] = alloc<R>(nfield_);
    for (int f = 0; f < 4; ++f) wall_[f] = alloc<R>(kp_.plane * cap_);
    conv_rows_ = convec_rows_enabled(d_.p.precision);
    if (!conv_rows_)
      for (int f = 0; f < 6; ++f) big_[f] = alloc<R>(kp_.istride_big * cap_);
    vol1_s_ = (long long)nz * ny * d_.K;
    vol1_b_ = (long long)nz * d_.ny2 * d_.K;
    const long long pl_s = (long long)ny * d_.K;
    specA_ = alloc<T2>(std::max({21 * vol1_s_, 6 * vol1_s_, 3 * vol1_b_}) * cap_);
    specB_ = alloc<T2>(std::max({42 * vol1_s_, 6 * vol1_b_, 9 * vol1_s_}) * cap_);
    specC_ = alloc<T2>(4LL * pl_s * cap_);
    // the convective term's own spectra: it runs beside the stress
    // divergence (and the Lagrangian update) in the fused step
    cvA_ = alloc<T2>(std::max(6 * vol1_s_, 3 * vol1_b_) * cap_);
    cvB_ = alloc<T2>(std::max(6 * vol1_b_, 3 * vol1_s_) * cap_);
    CK(cudaStreamCreateWithFlags(&st2_, cudaStreamNonBlocking));
    for (auto& e : ev_) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    hspec_ = alloc<double2>(3 * vol1_s_ * cap_);
    hplane_ = alloc<double2>(2 * pl_s * cap_);
    phat_ = alloc<double2>((nz + 1) * pl_s * cap_);
    build_thomas_pivots();
    err_ = alloc<int>(2);   // [0] zero pivot, [1] a bulk-copy wait that gave up
    zo_d_ = alloc<double>(cap_);
    flags_d_ = alloc<int>(cap_);
    // pinned staging ring for the per-step uploads (flags, averaging actions):
    // copies from pageable memory would wait for the stream every step
    CK(cudaMallocHost(&ring_h_, (size_t)kRing * cap_ * sizeof(int)));
    for (auto& e : ring_ev_) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    kp_.zo_i = zo_d_;
    kp_.iflags = flags_d_;
    sc_d_ = alloc<double>((long long)SC_N * cap_);
    cflmax_d_ = alloc<unsigned long long>(3LL * cap_);
    tact_d_ = alloc<int>(cap_);
    kp_.sc = sc_d_;
    // LESGO_GRAPHS=0 replays nothing: every step launches eagerly
    if (const char* g = std::getenv("LESGO_GRAPHS")) graphs_allowed_ = std::strcmp(g, "0") != 0;
    if (const char* b = std::getenv("LESGO_BRANCHES")) branches_allowed_ = std::strcmp(b, "0") != 0;
    if (const char* e = std::getenv("LESGO_XTARGET")) xtarget_ = std::max(256, std::atoi(e));
    if (const char* e = std::getenv("LESGO_YBUDGET")) ybudget_ = (size_t)std::max(8192, std::atoi(e));
    if (const char* e = std::getenv("LESGO_YTHREADS")) ythreads_ = std::atoi(e) == 128 ? 128 : 256;
    if (const char* e = std::getenv("LESGO_YSHORTCUT")) yshort_ = std::strcmp(e, "0") != 0;
    if (const char* e = std::getenv("LESGO_THOMAS"))
      thomas_mode_ = std::strcmp(e, "seq") == 0 ? 1 : std::strcmp(e, "seg") == 0 ? 2 : 0;
    use_graphs_ = graphs_allowed_;
    build_tables();
    // x-direction forward transforms as tensor-core GEMMs (FP32 transforms,
    // nx a multiple of 16 up to 128): LESGO_XDFT=1
    if (std::is_same<A, float>::value && nx % 16 == 0 && nx <= 128)
      if (const char* e = std::getenv("LESGO_XDFT"); e && std::strcmp(e, "1") == 0) {
        const std::vector<float> img = xdft_image(nx);
        xdft_w_ = alloc<float>((long long)img.size());
        CK(cudaMemcpyAsync(xdft_w_, img.data(), img.size() * sizeof(float), cudaMemcpyHostToDevice, st_));
      }
    CK(cudaStreamSynchronize(st_));
  }

  ~Solver() override {
    if (tri_gam_) cudaFree(tri_gam_);
    for (auto& r : prof_) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
    for (void* p : allocs_) cudaFree(p);
    for (void* p : turb_allocs_) cudaFree(p);
    for (auto& e : ev_)
      if (e) cudaEventDestroy(e);
    for (auto& e : ring_ev_)
      if (e) cudaEventDestroy(e);
    if (ring_h_) cudaFreeHost(ring_h_);
    if (st2_) cudaStreamDestroy(st2_);
    if (st_) cudaStreamDestroy(st_);
  }

  const Derived& der() const override { return d_; }
  int capacity() const override { return cap_; }
  int active() const override { return (int)slots_.size(); }

  // ---------------- instances --------------------------------------------------
  int add_instance(const InstanceSpec& spec) override {
    if ((int)slots_.size() >= cap_) throw Error(LESGO_ERR_NOMEM, "no free slot in this batch");
    if (!(spec.zo > 0)) throw Error(LESGO_ERR_ARG, "zo must be positive");
    Slot sl;
    sl.id = next_id_++;
    sl.spec = spec;
    sl.initu = d_.p.initu != 0;
    const int slot = (int)slots_.size();
    slots_.push_back(sl);
    sync_instance_params();
    if (!spec.turbines.empty() || kp_.turbines) rebuild_turbines(-1, -1);
    // fresh state: zero every field of the slot, then the seeded IC
    for (int f = 0; f < LESGO_NFIELDS; ++f)
      CK(cudaMemsetAsync(F_[f] + slot * kp_.istride, 0, kp_.istride * sizeof(R), st_));
    init_step_constants(slot);
    ic_slot(slot, spec.seed);
    CK(cudaStreamSynchronize(st_));
    return sl.id;
  }

  void remove_instance(int id) override {
    const int slot = slot_of(id);
    const int last = (int)slots_.size() - 1;
    if (slot != last) {
      // move the last instance into the freed slot (fields and its state)
      for (int f = 0; f < LESGO_NFIELDS; ++f)
        CK(cudaMemcpyAsync(F_[f] + slot * kp_.istride, F_[f] + last * kp_.istride, kp_.istride * sizeof(R),
                           cudaMemcpyDeviceToDevice, st_));
      CK(cudaMemcpyAsync(sc_d_ + (long long)slot * SC_N, sc_d_ + (long long)last * SC_N, SC_N * sizeof(double),
                         cudaMemcpyDeviceToDevice, st_));
      if (dlog_)
        CK(cudaMemcpyAsync(dlog_ + (long long)slot * dlog_cap_ * 6, dlog_ + (long long)last * dlog_cap_ * 6,
                           (size_t)dlog_cap_ * 6 * sizeof(double), cudaMemcpyDeviceToDevice, st_));
      if (tacc_)
        for (int f = 0; f < TA_N; ++f)
          CK(cudaMemcpyAsync(tacc_ + f * tacc_stride_ + slot * kp_.istride, tacc_ + f * tacc_stride_ + last * kp_.istride,
                             kp_.istride * sizeof(double), cudaMemcpyDeviceToDevice, st_));
      slots_[slot] = slots_[last];
    }
    const bool had_turbines = kp_.turbines != 0;
    slots_.pop_back();
    sync_instance_params();
    if (had_turbines) rebuild_turbines(slot, last);
    CK(cudaStreamSynchronize(st_));
  }

  // ---------------- field access -----------------------------------------
  void check_range(int f, int lbz, int nzhi) const {
    if (f < 0 || f >= LESGO_NFIELDS) throw Error(LESGO_ERR_ARG, "bad field id");
    if (lbz < 0 || nzhi > d_.nz || nzhi < lbz) throw Error(LESGO_ERR_ARG, "levels outside 0..nz");
  }
  void set_field(int id, int f, const double* h, int lbz, int nzhi, bool wait = true) override {
    check_range(f, lbz, nzhi);
    const int slot = slot_of(id);
    const long long n = (long long)(nzhi - lbz + 1) * kp_.plane;
    R* dst = F_[f] + slot * kp_.istride + (long long)lbz * kp_.plane;
    if (std::is_same<R, double>::value) {
      CK(cudaMemcpyAsync(dst, h, n * sizeof(double), cudaMemcpyHostToDevice, st_));
    } else {
      double* stg = staging(n);
      CK(cudaMemcpyAsync(stg, h, n * sizeof(double), cudaMemcpyHostToDevice, st_));
      k_convert<double, R><<<grid1(n), 256, 0, st_>>>(stg, dst, n);
      post();
    }
    if (wait) CK(cudaStreamSynchronize(st_));
  }
  void get_field(int id, int f, double* h, int lbz, int nzhi, bool wait = true) override {
    check_range(f, lbz, nzhi);
    const int slot = slot_of(id);
    const long long n = (long long)(nzhi - lbz + 1) * kp_.plane;
    const R* src = F_[f] + slot * kp_.istride + (long long)lbz * kp_.plane;
    if (std::is_same<R, double>::value) {
      CK(cudaMemcpyAsync(h, src, n * sizeof(double), cudaMemcpyDeviceToHost, st_));
    } else {
      double* stg = staging(n);
      k_convert<R, double><<<grid1(n), 256, 0, st_>>>(src, stg, n);
      post();
      CK(cudaMemcpyAsync(h, stg, n * sizeof(double), cudaMemcpyDeviceToHost, st_));
    }
    if (wait) CK(cudaStreamSynchronize(st_));
  }

  void init_ic(int id, uint64_t seed) override {
    const int slot = slot_of(id);
    slots_[slot].spec.seed = seed;
    ic_slot(slot, seed);
    CK(cudaStreamSynchronize(st_));
  }

  // ---------------- stage entry points (all active instances) -----------------
  void filt_da(int f, int fx, int fy) override {
    need_active();
    const R sc = (R)(1.0 / ((double)d_.nx * d_.ny));
    SrcFields<R, 1> src{{F_[f]}, sc, 1, 1, d_.ld, kp_.plane, imf(d_.nz)};
    xfwd<1>(src, d_.nx, d_.ny, d_.nz, specA_, px_);
    ypass_lin<1, 3, true, true, T2, T2>(specA_, 0, 1, d_.nz, d_.ny, specB_, d_.ny, d_.nz, 1, ROW_SAME,
                                        {{MUL_ONE}, {MUL_IKX}, {MUL_IKY}});
    DstFields<R, 3> dst{{F_[f], F_[fx], F_[fy]}, 1, 1, d_.ld, kp_.plane, imf(d_.nz)};
    xinv<3>(dst, specB_, d_.nx, d_.ny, d_.nz, px_);
  }
  void ddxy(int f, int fx, int fy) override {
    need_active();
    const R sc = (R)(1.0 / ((double)d_.nx * d_.ny));
    SrcFields<R, 1> src{{F_[f]}, sc, 1, 1, d_.ld, kp_.plane, imf(d_.nz)};
    xfwd<1>(src, d_.nx, d_.ny, d_.nz, specA_, px_);
    if (fx >= 0 && fy >= 0) {
      ypass_lin<1, 2, true, true, T2, T2>(specA_, 0, 1, d_.nz, d_.ny, specB_, d_.ny, d_.nz, 1, ROW_SAME,
                                          {{MUL_IKX}, {MUL_IKY}});
      DstFields<R, 2> dst{{F_[fx], F_[fy]}, 1, 1, d_.ld, kp_.plane, imf(d_.nz)};
      xinv<2>(dst, specB_, d_.nx, d_.ny, d_.nz, px_);
    } else {
      ypass_lin<1, 1, true, true, T2, T2>(specA_, 0, 1, d_.nz, d_.ny, specB_, d_.ny, d_.nz, 1, ROW_SAME,
                                          {{fx >= 0 ? MUL_IKX : MUL_IKY}});
      DstFields<R, 1> dst{{F_[fx >= 0 ? fx : fy]}, 1, 1, d_.ld, kp_.plane, imf(d_.nz)};
      xinv<1>(dst, specB_, d_.nx, d_.ny, d_.nz, px_);
    }
  }
  void ddz(int f, int dfdz, bool uv) override {
    need_active();
    const long long n = (long long)d_.nx * d_.ny * d_.nz * kp_.ninst;
    if (uv) k_ddz<R, true><<<grid1(n), 256, 0, st_>>>(F_[f], F_[dfdz], kp_);
    else k_ddz<R, false><<<grid1(n), 256, 0, st_>>>(F_[f], F_[dfdz], kp_);
    post();
  }
  void test_filter(int f, int level) override {
    need_active();
    if (level < 0 || level > d_.nz) throw Error(LESGO_ERR_ARG, "level");
    // in place: output planes are the level's planes (instance stride = field stride)
    filter_planes(F_[f], F_[f], level, F_[f] + (long long)level * kp_.plane, F_[f] + (long long)level * kp_.plane,
                  1, kp_.istride);
  }
  void wallstress() override {
    need_active();
    wall_planes();
    const int n = d_.nx * d_.ny;
    k_wall<R><<<dim3((n + 255) / 256, kp_.ninst), 256, 0, st_>>>(F_[LESGO_U], F_[LESGO_V], wall_[0], wall_[1], wall_[2],
                                                                wall_[3], F_[LESGO_TXZ], F_[LESGO_TYZ], F_[LESGO_DUDZ],
                                                                F_[LESGO_DVDZ], kp_);
    post();
  }
  void sgs_stag() override {
    need_active();
    bool lag_any = false;
    for (const auto& sl : slots_) lag_any = lag_any || (sl.flags & IF_LAG);
    if (!lag_any) {
      column<COL_STORE_S | COL_TAU>();
    } else {
      column<COL_STORE_S>();
      lagrange();
      column<COL_READ_S | COL_TAU>();
    }
    commit_lagrange_init();
  }
  void divstress(int which) override {
    need_active();
    const R sc = (R)(1.0 / ((double)d_.nx * d_.ny));
    const R idz = (R)(1.0 / d_.dz);
    const InstMap im = imf(d_.nz);
    if (which == 3) {
      SrcFields<R, 5> src{{F_[LESGO_TXX], F_[LESGO_TXY], F_[LESGO_TYY], F_[LESGO_TXZ], F_[LESGO_TYZ]}, sc, 1, 1, d_.ld,
                          kp_.plane, im};
      xfwd<5>(src, d_.nx, d_.ny, d_.nz, specA_, px_, "divstress.xfwd");
      ypass_lin<5, 3, true, true, T2, T2>(specA_, 0, 1, d_.nz, d_.ny, specB_, d_.ny, d_.nz, 1, ROW_SAME,
                                          {{MUL_IKX, MUL_IKY, 0, 0, 0}, {0, MUL_IKX, MUL_IKY, 0, 0}, {0, 0, 0, MUL_IKX, MUL_IKY}},
                                          "divstress.ypass");
      DstDiv<R, 3> dst{F_[LESGO_DIVTX], F_[LESGO_DIVTY], F_[LESGO_DIVTZ], F_[LESGO_TXZ], F_[LESGO_TYZ], F_[LESGO_TZZ],
                       idz, d_.ld, d_.nz, kp_.plane, im};
      xinv<3>(dst, specB_, d_.nx, d_.ny, d_.nz, px_, "divstress.xinv", 6);
    } else if (which == 1) {
      SrcFields<R, 3> src{{F_[LESGO_TXX], F_[LESGO_TXY], F_[LESGO_TYY]}, sc, 1, 1, d_.ld, kp_.plane, im};
      xfwd<3>(src, d_.nx, d_.ny, d_.nz, specA_, px_);
      ypass_lin<3, 2, true, true, T2, T2>(specA_, 0, 1, d_.nz, d_.ny, specB_, d_.ny, d_.nz, 1, ROW_SAME,
                                          {{MUL_IKX, MUL_IKY, 0}, {0, MUL_IKX, MUL_IKY}});
      DstDiv<R, 1> dst{F_[LESGO_DIVTX], F_[LESGO_DIVTY], F_[LESGO_DIVTZ], F_[LESGO_TXZ], F_[LESGO_TYZ], F_[LESGO_TZZ],
                       idz, d_.ld, d_.nz, kp_.plane, im};
      xinv<2>(dst, specB_, d_.nx, d_.ny, d_.nz, px_);
    } else {
      SrcFields<R, 2> src{{F_[LESGO_TXZ], F_[LESGO_TYZ]}, sc, 1, 1, d_.ld, kp_.plane, im};
      xfwd<2>(src, d_.nx, d_.ny, d_.nz, specA_, px_);
      ypass_lin<2, 1, true, true, T2, T2>(specA_, 0, 1, d_.nz, d_.ny, specB_, d_.ny, d_.nz, 1, ROW_SAME,
                                          {{MUL_IKX, MUL_IKY}});
      DstDiv<R, 2> dst{F_[LESGO_DIVTX], F_[LESGO_DIVTY], F_[LESGO_DIVTZ], F_[LESGO_TXZ], F_[LESGO_TYZ], F_[LESGO_TZZ],
                       idz, d_.ld, d_.nz, kp_.plane, im};
      xinv<1>(dst, specB_, d_.nx, d_.ny, d_.nz, px_);
    }
  }
  void convec() override { need_active(); convec_impl(false); }
  void turbines_forcing() override {
    need_active();
    if (!kp_.turbines) return;
    turb_impl();
  }
  void begin_step() override {
    need_active();
    advance_counters();
    bool lag_any = false;
    upload_flags(&lag_any);
    step_begin_kernels();
    for (int c = 0; c < 3; ++c)
      CK(cudaMemcpyAsync(F_[LESGO_RHSX_F + c], F_[LESGO_RHSX + c], kp_.istride * kp_.ninst * sizeof(R),
                         cudaMemcpyDeviceToDevice, st_));
  }
  void rhs_assemble() override {
    need_active();
    const long long n = kp_.plane * d_.nz * kp_.ninst;
    k_rhs_assemble<R><<<grid1(n), 256, 0, st_>>>(F_[LESGO_RHSX], F_[LESGO_RHSY], F_[LESGO_RHSZ], F_[LESGO_DIVTX],
                                                 F_[LESGO_DIVTY], F_[LESGO_DIVTZ], F_[LESGO_FXA], F_[LESGO_FYA],
                                                 F_[LESGO_FZA], kp_);
    post();
  }
  void ab2() override {
    need_active();
    for (int s = 0; s < (int)slots_.size(); ++s)
      if (slots_[s].jt_total == 1 && !slots_[s].initu)
        for (int c = 0; c < 3; ++c)
          CK(cudaMemcpyAsync(F_[LESGO_RHSX_F + c] + s * kp_.istride, F_[LESGO_RHSX + c] + s * kp_.istride,
                             kp_.istride * sizeof(R), cudaMemcpyDeviceToDevice, st_));
    const long long n = kp_.plane * d_.nz * kp_.ninst;
    k_ab2<R><<<grid1(n), 256, 0, st_>>>(F_[LESGO_U], F_[LESGO_V], F_[LESGO_W], F_[LESGO_RHSX], F_[LESGO_RHSY],
                                        F_[LESGO_RHSZ], F_[LESGO_RHSX_F], F_[LESGO_RHSY_F], F_[LESGO_RHSZ_F], kp_);
    post();
  }
  void press_stag_array() override { need_active(); pressure_impl(false); }
  void rhs_sub_dp() override {
    need_active();
    const long long n = kp_.plane * d_.nz * kp_.ninst;
    k_rhs_sub_dp<R><<<grid1(n), 256, 0, st_>>>(F_[LESGO_RHSX], F_[LESGO_RHSY], F_[LESGO_RHSZ], F_[LESGO_DPDX],
                                               F_[LESGO_DPDY], F_[LESGO_DPDZ], kp_);
    post();
  }
  void project() override {
    need_active();
    const long long n = (long long)d_.nx * d_.ny * d_.nz * kp_.ninst;
    k_project<R><<<grid1(n), 256, 0, st_>>>(F_[LESGO_DPDX], F_[LESGO_DPDY], F_[LESGO_DPDZ], F_[LESGO_U], F_[LESGO_V],
                                            F_[LESGO_W], kp_);
    post();
    k_project_bc<R><<<grid1(kp_.plane * kp_.ninst), 256, 0, st_>>>(F_[LESGO_U], F_[LESGO_V], F_[LESGO_W], kp_);
    post();
  }

  // ---------------- fused time loop ------------------------------------------
  void step(int nsteps) override {
    need_active();
    for (int s = 0; s < nsteps; ++s) {
      advance_counters();
      bool lag_any = false;
      const bool special = upload_flags(&lag_any);
      const int code = (lag_any ? 1 : 0) | (kp_.ninst << 1);
      if (!special && use_graphs_) {
        auto it = graphs_.find(code);
        if (it == graphs_.end()) {
          cudaGraph_t g;
          launches_ = 0;
          CK(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
          try {
            step_body(lag_any);
          } catch (...) {
            cudaStreamEndCapture(st_, &g);
            throw;
          }
          CK(cudaStreamEndCapture(st_, &g));
          cudaGraphExec_t ge;
          CK(cudaGraphInstantiate(&ge, g, 0));
          cudaGraphDestroy(g);
          graphs_[code] = ge;
          launch_count_[lag_any ? 1 : 0] = launches_;
          it = graphs_.find(code);
        }
        CK(cudaGraphLaunch(it->second, st_));
      } else {
        launches_ = 0;
        step_body(lag_any);
        if (!special) launch_count_[lag_any ? 1 : 0] = launches_;
      }
      commit_lagrange_init();
      if (tavg_on_) tavg_sample();
      if (dlog_every_) diag_log_sample();
    }
  }

  // ---------------- time averaging (time_average.f90, io.f90:557-580) --------
  void tavg_config(int nstart, int nend, int nskip) override {
    if (nskip < 1 || nend < nstart) throw Error(LESGO_ERR_ARG, "tavg: need nskip >= 1 and nend >= nstart");
    if (!tacc_) {
      tacc_stride_ = kp_.istride * cap_;
      tacc_ = alloc<double>(TA_N * tacc_stride_);
      tw_d_ = alloc<double>(cap_);
    }
    CK(cudaMemsetAsync(tacc_, 0, TA_N * tacc_stride_ * sizeof(double), st_));
    ta_nstart_ = nstart; ta_nend_ = nend; ta_nskip_ = nskip;
    tavg_on_ = true;
    for (size_t s = 0; s < slots_.size(); ++s) {
      slots_[s].ta_init = false;
      write_sc((int)s, SC_TAW, 0.0);
      write_sc((int)s, SC_TAT, 0.0);
    }
    CK(cudaStreamSynchronize(st_));
  }
  // output_loop's schedule for each instance after a step: every step of
  // [nstart, nend] adds dt; the first sample step starts the sums, later ones
  // add the fields weighted by the time since the previous sample.
  void tavg_sample() override {
    if (!tavg_on_) throw Error(LESGO_ERR_ARG, "tavg: not configured");
    need_active();
    // act: 0 nothing, 1 tavg%init, 2 tavg%init from tavg.out, 3 tavg%compute;
    // the pending weight (dt summed over the window's steps) lives on the device
    std::vector<int> act(slots_.size(), 0);
    bool any = false, sample = false;
    for (size_t s = 0; s < slots_.size(); ++s) {
      Slot& sl = slots_[s];
      if (sl.jt_total < ta_nstart_ || sl.jt_total > ta_nend_) continue;
      if ((sl.jt_total - ta_nstart_) % ta_nskip_ != 0) continue;
      any = true;
      if (!sl.ta_init) {
        // zero the sums, or keep those read from tavg.out (which carries no
        // pressure sum: time_average.f90:114-150)
        for (int f = 0; f < TA_N; ++f)
          if (!sl.ta_loaded || f == TA_P)
            CK(cudaMemsetAsync(tacc_ + f * tacc_stride_ + s * kp_.istride, 0, kp_.istride * sizeof(double), st_));
        act[s] = sl.ta_loaded ? 2 : 1;
        sl.ta_init = true;
        sl.ta_loaded = false;
      } else {
        act[s] = 3;
        sample = true;
      }
    }
    if (!any) return;
    upload_ints(tact_d_, act);
    pre();
    k_tavg_prep<<<(kp_.ninst + 63) / 64, 64, 0, st_>>>(sc_d_, tact_d_, tw_d_, kp_.ninst);
    post("tavg.prep", 0.0);
    if (!sample) return;
    TavgArgs<R> a;
    a.u = F_[LESGO_U]; a.v = F_[LESGO_V]; a.w = F_[LESGO_W]; a.p = F_[LESGO_P];
    a.txx = F_[LESGO_TXX]; a.tyy = F_[LESGO_TYY]; a.tzz = F_[LESGO_TZZ];
    a.txy = F_[LESGO_TXY]; a.txz = F_[LESGO_TXZ]; a.tyz = F_[LESGO_TYZ];
    a.fxa = F_[LESGO_FXA]; a.fya = F_[LESGO_FYA]; a.fza = F_[LESGO_FZA]; a.cs = F_[LESGO_CS_OPT2];
    a.dudy = F_[LESGO_DUDY]; a.dudz = F_[LESGO_DUDZ]; a.dvdx = F_[LESGO_DVDX]; a.dvdz = F_[LESGO_DVDZ];
    a.dwdx = F_[LESGO_DWDX]; a.dwdy = F_[LESGO_DWDY];
    a.acc = tacc_; a.acc_stride = tacc_stride_; a.wgt = tw_d_; a.kp = kp_;
    const long long n = (long long)d_.nx * d_.ny * d_.nz * kp_.ninst;
    pre();
    k_tavg<R><<<grid1(n), 256, 0, st_>>>(a);
    post("tavg.compute", (double)n * (20.0 * sizeof(R) + 2.0 * TA_N * 8));
  }
  void tavg_get(int id, int which, double* host, int lbz, int nzhi) override {
    if (!tacc_) throw Error(LESGO_ERR_ARG, "tavg: not configured");
    if (which < 0 || which >= TA_N + 6) throw Error(LESGO_ERR_ARG, "tavg: bad quantity");
    if (lbz < 0 || nzhi > d_.nz || nzhi < lbz) throw Error(LESGO_ERR_ARG, "levels outside 0..nz");
    const int slot = slot_of(id);
    const double tot = read_sc(slot, SC_TAT);
    if (!(tot > 0)) throw Error(LESGO_ERR_ARG, "tavg: no sample yet");
    double* stg = staging(kp_.istride);
    const long long n = kp_.istride;
    k_tavg_get<<<grid1(n), 256, 0, st_>>>(tacc_, tacc_stride_, slot * kp_.istride, which, 1.0 / tot, stg, n);
    post();
    const long long off = (long long)lbz * kp_.plane, cnt = (long long)(nzhi - lbz + 1) * kp_.plane;
    CK(cudaMemcpyAsync(host, stg + off, cnt * sizeof(double), cudaMemcpyDeviceToHost, st_));
    CK(cudaStreamSynchronize(st_));
  }
  void tavg_profile(int id, int which, double* prof, int n) override {
    if (n < d_.nz + 1) throw Error(LESGO_ERR_ARG, "tavg_profile: need nz+1 values");
    if (!tacc_) throw Error(LESGO_ERR_ARG, "tavg: not configured");
    if (which < 0 || which >= TA_N + 6) throw Error(LESGO_ERR_ARG, "tavg: bad quantity");
    const int slot = slot_of(id);
    const double tot = read_sc(slot, SC_TAT);
    if (!(tot > 0)) throw Error(LESGO_ERR_ARG, "tavg: no sample yet");
    double* stg = staging(kp_.istride);
    if (!prof_d_) prof_d_ = alloc<double>(d_.nz + 1);
    k_tavg_get<<<grid1(kp_.istride), 256, 0, st_>>>(tacc_, tacc_stride_, slot * kp_.istride, which, 1.0 / tot,
                                                    stg, kp_.istride);
    post();
    k_plane_mean<<<d_.nz + 1, 256, 0, st_>>>(stg, d_.nx, d_.ny, d_.ld, prof_d_);
    post();
    CK(cudaMemcpyAsync(prof, prof_d_, (d_.nz + 1) * sizeof(double), cudaMemcpyDeviceToHost, st_));
    CK(cudaStreamSynchronize(st_));
  }
  double tavg_total_time(int id) override { return read_sc(slot_of(id), SC_TAT); }
  double sim_time(int id) override { return read_sc(slot_of(id), SC_TIME); }
  double time_step(int id) override { return read_sc(slot_of(id), SC_DT); }

  // ---------------- checkpoint / restart (io.f90:1173-1267, initial.f90:20-380) ----
  // The 11 fields of vel.out in record order.
  static constexpr int kVelFields[11] = {LESGO_U,    LESGO_V,    LESGO_W,    LESGO_RHSX, LESGO_RHSY, LESGO_RHSZ,
                                         LESGO_CS_OPT2, LESGO_F_LM, LESGO_F_MM, LESGO_F_QN, LESGO_F_NN};
  // tavg.out's 25 sums in record order (the pressure sum is not written).
  static constexpr int kTavgFile[25] = {TA_U,   TA_V,   TA_W,   TA_U_W, TA_V_W, TA_W_UV, TA_U2,  TA_V2,  TA_W2,
                                        TA_UV,  TA_UW,  TA_VW,  TA_TXX, TA_TYY, TA_TZZ,  TA_TXY, TA_TXZ, TA_TYZ,
                                        TA_FX,  TA_FY,  TA_FZ,  TA_CS,  TA_VORTX, TA_VORTY, TA_VORTZ};

  void checkpoint_write(int id, const std::string& pre, int mpi_names) override {
    const int slot = slot_of(id);
    Slot& sl = slots_[slot];
    const std::string sfx = mpi_names ? ".c0" : "";
    const long long pl = kp_.plane * d_.nz;
    std::vector<double> buf(11 * pl);
    for (int i = 0; i < 11; ++i) get_field(id, kVelFields[i], buf.data() + i * pl, 1, d_.nz);
    try {
      {
        fio::File fl(pre + "vel.out" + sfx, "wb");
        if (!fl.f) throw fio::IoError{"cannot open " + pre + "vel.out" + sfx};
        fio::write_record(fl.f, {{buf.data(), (int64_t)buf.size() * 8}});
      }
      fio::GridOut go;
      go.nproc = 1; go.nx = d_.nx; go.ny = d_.ny; go.nz = d_.nz;
      go.Lx = d_.p.L_x; go.Ly = d_.p.L_y; go.Lz = d_.p.L_z;
      fio::write_grid(pre + "grid.out", go);
      if (sl.ta_init) {
        // sums of x < nx at levels 1..nz, (nx, ny, nz) like the reference
        fio::File fl(pre + "tavg.out" + sfx, "wb");
        if (!fl.f) throw fio::IoError{"cannot open " + pre + "tavg.out" + sfx};
        const double tat = read_sc(slot, SC_TAT);
        fio::write_record(fl.f, {{&tat, 8}});
        std::vector<double> lev(pl), pk((size_t)d_.nx * d_.ny * d_.nz);
        for (int q : kTavgFile) {
          CK(cudaMemcpyAsync(lev.data(), tacc_ + q * tacc_stride_ + slot * kp_.istride + kp_.plane, pl * sizeof(double),
                             cudaMemcpyDeviceToHost, st_));
          CK(cudaStreamSynchronize(st_));
          for (int k = 0; k < d_.nz; ++k)
            for (int j = 0; j < d_.ny; ++j)
              std::memcpy(&pk[((size_t)k * d_.ny + j) * d_.nx], &lev[(size_t)k * kp_.plane + (size_t)j * d_.ld],
                          d_.nx * sizeof(double));
          fio::write_record(fl.f, {{pk.data(), (int64_t)pk.size() * 8}});
        }
      }
      // cfl written: the CFL number of a varying step, else the current maximum
      double dg[4];
      diag(id, dg);
      fio::TimeDat td;
      const double t = read_sc(slot, SC_TIME);
      td.jt_total = sl.jt_total;
      td.total_time = t;
      td.total_time_dim = read_sc(slot, SC_TDIM);
      td.dt = read_sc(slot, SC_DT);
      td.cfl = d_.p.use_cfl_dt ? d_.p.cfl : dg[2];
      fio::write_time(pre + "total_time.dat", td);
    } catch (const fio::IoError& e) {
      throw Error(LESGO_ERR_ARG, "checkpoint: " + e.msg);
    }
  }

  // Returns 1 when the checkpoint was of this grid (initu: every field of
  // vel.out taken, no Euler first step, no Lagrangian initialisation), 0 when
  // u, v, w were interpolated from another grid (initial.f90:242-380; the
  // other fields start from zero).
  int checkpoint_read(int id, const std::string& pre) override {
    const int slot = slot_of(id);
    Slot& sl = slots_[slot];
    const long long pl = kp_.plane * d_.nz;
    int exact = 0;
    try {
      bool interp = false;
      fio::GridOut g;
      g.nproc = 1; g.nx = d_.nx; g.ny = d_.ny; g.nz = d_.nz;
      g.Lx = d_.p.L_x; g.Ly = d_.p.L_y; g.Lz = d_.p.L_z;
      if (fio::exists(pre + "grid.out")) {
        g = fio::read_grid(pre + "grid.out");
        interp = !(g.nproc == 1 && g.nx == d_.nx && g.ny == d_.ny && g.nz == d_.nz && g.Lx == d_.p.L_x &&
                   g.Ly == d_.p.L_y && g.Lz == d_.p.L_z);
      }
      std::vector<char> rec;
      if (!interp) {
        std::string name = pre + "vel.out";
        if (!fio::exists(name)) name += ".c0";
        fio::File fl(name, "rb");
        if (!fl.f) throw fio::IoError{"no checkpoint at " + pre + "vel.out"};
        if (!fio::read_record(fl.f, rec) || (long long)rec.size() != 11 * pl * 8)
          throw fio::IoError{name + ": record is not 11 fields of (ld, ny, 1:nz)"};
        for (int i = 0; i < 11; ++i)
          set_field(id, kVelFields[i], reinterpret_cast<const double*>(rec.data()) + i * pl, 1, d_.nz);
        exact = 1;
      } else {
        if (g.nproc < 1 || g.nx < 2 || g.ny < 1 || g.nz < 2) throw fio::IoError{"grid.out: bad grid"};
        const int ld_f = 2 * (g.nx / 2 + 1);
        const int nzt = (g.nz - 1) * g.nproc + 1;
        const long long pf = (long long)ld_f * g.ny;
        std::vector<double> uvw[3];
        for (auto& a : uvw) a.assign((size_t)pf * nzt, 0.0);
        for (int c = 0; c < g.nproc; ++c) {
          std::string name = pre + "vel.out" + (g.nproc > 1 ? ".c" + std::to_string(c) : "");
          if (g.nproc == 1 && !fio::exists(name)) name += ".c0";
          fio::File fl(name, "rb");
          if (!fl.f) throw fio::IoError{"cannot open " + name};
          if (!fio::read_record(fl.f, rec) || (long long)rec.size() < 3 * pf * g.nz * 8)
            throw fio::IoError{name + ": record shorter than u, v, w of grid.out's grid"};
          // rank c holds global levels c (nz - 1) + 1 .. c (nz - 1) + nz
          for (int f = 0; f < 3; ++f)
            std::memcpy(uvw[f].data() + (size_t)c * (g.nz - 1) * pf,
                        rec.data() + (size_t)f * pf * g.nz * 8, (size_t)pf * g.nz * 8);
        }
        fio::Regrid rg{g.nx, g.ny, nzt, ld_f, g.Lx, g.Ly, g.Lz, d_.nx, d_.ny, d_.nz, d_.ld, d_.dx, d_.dy, d_.dz};
        std::vector<double> out[3];
        for (auto& a : out) a.assign((size_t)pl, 0.0);
        rg.apply(uvw[0].data(), uvw[1].data(), uvw[2].data(), out[0].data(), out[1].data(), out[2].data());
        std::vector<double> zero((size_t)pl, 0.0);
        for (int i = 0; i < 11; ++i)
          set_field(id, kVelFields[i], i < 3 ? out[i].data() : zero.data(), 1, d_.nz);
      }
      sl.initu = exact != 0;
      sl.jt = 0;
      sl.flm_init = sl.fqn_init = false;
      sl.lag_prev = false;
      init_step_constants(slot);
      if (fio::exists(pre + "total_time.dat")) {
        // io.f90:73-96: counters and time; with use_cfl_dt also the last dt
        const fio::TimeDat t = fio::read_time(pre + "total_time.dat");
        sl.jt_total = (int)t.jt_total;
        write_sc(slot, SC_TIME, t.total_time);
        write_sc(slot, SC_TDIM, t.total_time_dim);
        if (d_.p.use_cfl_dt && t.dt > 0) write_sc(slot, SC_DT, t.dt);
      } else {
        sl.jt_total = 0;
      }
      // time-averaging restart (time_average.f90:114-150)
      std::string tname = pre + "tavg.out";
      if (!fio::exists(tname)) tname += ".c0";
      if (tavg_on_ && fio::exists(tname)) {
        fio::File fl(tname, "rb");
        std::vector<char> r;
        if (!fio::read_record(fl.f, r) || r.size() != 8) throw fio::IoError{tname + ": no total_time record"};
        double tat = 0.0;
        std::memcpy(&tat, r.data(), 8);
        write_sc(slot, SC_TAT, tat);
        write_sc(slot, SC_TAW, 0.0);
        const size_t n3 = (size_t)d_.nx * d_.ny * d_.nz;
        std::vector<double> lev((size_t)pl, 0.0);
        for (int q : kTavgFile) {
          if (!fio::read_record(fl.f, r) || r.size() != n3 * 8) throw fio::IoError{tname + ": bad sum record"};
          const double* src = reinterpret_cast<const double*>(r.data());
          for (int k = 0; k < d_.nz; ++k)
            for (int j = 0; j < d_.ny; ++j)
              std::memcpy(&lev[(size_t)k * kp_.plane + (size_t)j * d_.ld], src + ((size_t)k * d_.ny + j) * d_.nx,
                          d_.nx * sizeof(double));
          CK(cudaMemcpyAsync(tacc_ + q * tacc_stride_ + slot * kp_.istride + kp_.plane, lev.data(),
                             pl * sizeof(double), cudaMemcpyHostToDevice, st_));
          CK(cudaStreamSynchronize(st_));
        }
        sl.ta_loaded = true;
        sl.ta_init = false;
      }
    } catch (const fio::IoError& e) {
      throw Error(LESGO_ERR_ARG, "restart: " + e.msg);
    }
    return exact;
  }

  int sync() override {
    CK(cudaStreamSynchronize(st_));
    int e[2] = {0, 0};
    CK(cudaMemcpy(e, err_, 2 * sizeof(int), cudaMemcpyDeviceToHost));
    if (e[1]) {
      CK(cudaMemset(err_ + 1, 0, sizeof(int)));
      throw Error(LESGO_ERR_CUDA, "a bulk copy into shared memory did not complete within its wait limit");
    }
    if (e[0]) {
      CK(cudaMemset(err_, 0, sizeof(int)));
      return LESGO_ERR_NUMERIC;
    }
    return LESGO_OK;
  }

  void diag(int id, double* out) override {
    const int slot = slot_of(id);
    const int nb = 4 * 152;
    if (!diag_part_) { diag_part_ = alloc<double>(nb * 7); diag_out_ = alloc<double>(8); }
    k_diag<R><<<nb, 256, 0, st_>>>(F_[LESGO_DUDX], F_[LESGO_DVDY], F_[LESGO_DWDZ], F_[LESGO_U], F_[LESGO_V], F_[LESGO_W],
                                   F_[LESGO_TXZ], F_[LESGO_TYZ], kp_, diag_part_, slot);
    post();
    k_diag_final<<<1, 32, 0, st_>>>(diag_part_, nb, diag_out_);
    post();
    double h[7];
    CK(cudaMemcpyAsync(h, diag_out_, 7 * sizeof(double), cudaMemcpyDeviceToHost, st_));
    CK(cudaStreamSynchronize(st_));
    const double npts = (double)d_.nx * d_.ny * (d_.nz - 1);
    out[0] = h[0] / npts;
    out[1] = h[1] * 0.5 / npts;
    out[2] = read_sc(slot, SC_DT) * std::max({h[2] / d_.dx, h[3] / d_.dy, h[4] / d_.dz});
    const double nxy = (double)d_.nx * d_.ny;
    out[3] = std::sqrt((h[5] / nxy) * (h[5] / nxy) + (h[6] / nxy) * (h[6] / nxy));
  }

  // ---------------- tile-shape autotuner ----------------------------------------
  // Picks the tile shapes of the transform passes (complex values per block
  // of the x passes, shared memory per block of the y passes) by timing this
  // handle's own fused step at every candidate: the fields, step constants
  // and disk states are copied aside, a normal step, a second normal step and
  // a step with the dynamic update run eagerly per candidate, and the copy is
  // put back, so the simulation state is unchanged (tile shapes do not change
  // results).  Without memory for the copy, the passes are timed alone on
  // scratch buffers instead.
  void autotune(int* xt_out, int* yb_out) override {
    need_active();
    const size_t fbytes = (size_t)nfield_ * sizeof(R);
    const size_t sbytes = (size_t)SC_N * cap_ * sizeof(double);
    const size_t tbytes = kp_.turbines ? 3 * (size_t)th_.n * sizeof(double) : 0;
    unsigned char* snap = nullptr;
    if (cudaMalloc(&snap, fbytes * LESGO_NFIELDS + sbytes + tbytes) != cudaSuccess) {
      cudaGetLastError();
      autotune_passes();
    } else {
      auto save = [&](bool back) {
        unsigned char* q = snap;
        auto mv = [&](void* dev, size_t n) {
          CK(cudaMemcpyAsync(back ? dev : (void*)q, back ? (const void*)q : dev, n, cudaMemcpyDeviceToDevice, st_));
          q += n;
        };
        for (int f = 0; f < LESGO_NFIELDS; ++f) mv(F_[f], fbytes);
        mv(sc_d_, sbytes);
        if (tbytes) { mv(td_.u_d, tbytes / 3); mv(td_.u_d_T, tbytes / 3); mv(td_.f_n, tbytes / 3); }
      };
      save(false);
      cudaEvent_t e0, e1;
      CK(cudaEventCreate(&e0));
      CK(cudaEventCreate(&e1));
      // every shape timed in three interleaved rounds (the fastest round
      // counts); a shape replaces the default one only when it is more than
      // 2 % faster, since the handle's steps will also run beside other
      // handles' and single timings vary by about that much
      struct Cand { int xt; size_t yb; float ms; };
      std::vector<Cand> cands;
      for (int xt : {1024, 2048, 4096})
        for (size_t yb : {(size_t)32768, (size_t)49152, (size_t)65536, (size_t)112640}) cands.push_back({xt, yb, 1e30f});
      const int x0 = xtarget_;
      const size_t y0 = ybudget_;
      for (int round = 0; round < 3; ++round)
        for (auto& cd : cands) {
          xtarget_ = cd.xt;
          ybudget_ = cd.yb;
          step_body(false);   // sets the kernels' shared-memory limits at this shape
          CK(cudaEventRecord(e0, st_));
          step_body(false);
          step_body(false);
          step_body(true);
          CK(cudaEventRecord(e1, st_));
          CK(cudaEventSynchronize(e1));
          float ms = 0.f;
          CK(cudaEventElapsedTime(&ms, e0, e1));
          cd.ms = std::min(cd.ms, ms);
        }
      const Cand* best = &cands[0];
      const Cand* dflt = nullptr;
      for (const auto& cd : cands) {
        if (cd.ms < best->ms) best = &cd;
        if (cd.xt == x0 && cd.yb == y0) dflt = &cd;
      }
      if (dflt && best->ms > 0.98f * dflt->ms) best = dflt;
      xtarget_ = best->xt;
      ybudget_ = best->yb;
      save(true);
      CK(cudaStreamSynchronize(st_));
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      cudaFree(snap);
    }
    graphs_clear();   // tile shapes are part of the captured launches
    if (xt_out) *xt_out = xtarget_;
    if (yb_out) *yb_out = (int)ybudget_;
  }
  // The fallback: the three pass kinds timed alone on scratch buffers (6
  // fields forward from the fields and inverse into the 3/2-grid scratch;
  // 1 -> 3 and 5 -> 3 y passes on scratch spectra).
  void autotune_passes() {
    const int nz = d_.nz, ny = d_.ny;
    const InstMap im = imf(nz);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    auto timed = [&](auto&& fn) {
      fn();
      CK(cudaEventRecord(e0, st_));
      for (int r = 0; r < 3; ++r) fn();
      CK(cudaEventRecord(e1, st_));
      CK(cudaEventSynchronize(e1));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      return ms;
    };
    const R sc = (R)(1.0 / ((double)d_.nx * ny));
    float best = 1e30f;
    int best_x = xtarget_;
    for (int xt : {1024, 2048, 4096}) {
      xtarget_ = xt;
      const float ms = timed([&] {
        SrcFields<R, 6> src{{F_[LESGO_U], F_[LESGO_V], F_[LESGO_W], F_[LESGO_DUDX], F_[LESGO_DUDY], F_[LESGO_DUDZ]},
                            sc, 1, 1, d_.ld, kp_.plane, im};
        xfwd<6>(src, d_.nx, ny, nz, specA_, px_, "tune.xfwd");
        // into scratch only: the interpolation temporaries (free between
        // steps), two of them twice, which is the same work per launch
        DstFields<R, 6> dst{{Ftmp_[0], Ftmp_[1], Ftmp_[2], Ftmp_[3], Ftmp_[0], Ftmp_[1]}, 1, 1, d_.ld, kp_.plane, im};
        xinv<6>(dst, specA_, d_.nx, ny, nz, px_, "tune.xinv");
      });
      if (ms < best) { best = ms; best_x = xt; }
    }
    xtarget_ = best_x;
    best = 1e30f;
    size_t best_y = ybudget_;
    for (size_t yb : {(size_t)32768, (size_t)49152, (size_t)65536, (size_t)112640}) {
      ybudget_ = yb;
      const float ms = timed([&] {
        ypass_lin<1, 3, true, true, T2, T2>(specA_, 0, 1, nz, ny, specB_, ny, nz, 3, ROW_SAME,
                                            {{MUL_ONE}, {MUL_IKX}, {MUL_IKY}}, "tune.ypass13");
        ypass_lin<5, 3, true, true, T2, T2>(specA_, 0, 1, nz, ny, specB_, ny, nz, 1, ROW_SAME,
                                            {{MUL_IKX, MUL_IKY}, {MUL_ZERO, MUL_IKX, MUL_IKY}, {MUL_ZERO, MUL_ZERO,
                                             MUL_ZERO, MUL_IKX, MUL_IKY}}, "tune.ypass53");
      });
      if (ms < best) { best = ms; best_y = yb; }
    }
    ybudget_ = best_y;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }

  // ---------------- diagnostics log (main.f90:359-436: wbase / nenergy) -----
  void diag_log_config(int every, int capacity) override {
    if (every < 1 || capacity < 1) throw Error(LESGO_ERR_ARG, "diag log: every and capacity must be >= 1");
    if (!diag_part_) { diag_part_ = alloc<double>(4 * 152 * 7); diag_out_ = alloc<double>(8); }
    if (capacity != dlog_cap_) {
      if (dlog_) {   // queued samples may still write the old ring
        CK(cudaStreamSynchronize(st_));
        release(dlog_);
      }
      dlog_ = alloc<double>((long long)cap_ * capacity * 6);
      dlog_cap_ = capacity;
    }
    dlog_every_ = every;
    for (auto& sl : slots_) sl.dlog_count = 0;
  }
  // A row for every instance whose jt_total is a multiple of `every`.
  void diag_log_sample() override {
    if (!dlog_every_) throw Error(LESGO_ERR_ARG, "diag log: not configured");
    const int nb = 4 * 152;
    const double npts = (double)d_.nx * d_.ny * (d_.nz - 1), nxy = (double)d_.nx * d_.ny;
    for (size_t s = 0; s < slots_.size(); ++s) {
      Slot& sl = slots_[s];
      if (sl.jt_total % dlog_every_ != 0) continue;
      double* row = dlog_ + ((long long)s * dlog_cap_ + sl.dlog_count % dlog_cap_) * 6;
      pre();
      k_diag<R><<<nb, 256, 0, st_>>>(F_[LESGO_DUDX], F_[LESGO_DVDY], F_[LESGO_DWDZ], F_[LESGO_U], F_[LESGO_V],
                                     F_[LESGO_W], F_[LESGO_TXZ], F_[LESGO_TYZ], kp_, diag_part_, (int)s);
      post("diag.reduce", (double)kp_.plane * d_.nz * 8 * sizeof(R));
      pre();
      k_diag_log_final<<<1, 32, 0, st_>>>(diag_part_, nb, sc_d_ + (long long)s * SC_N, row, (double)sl.jt_total, npts,
                                          nxy, d_.dx, d_.dy, d_.dz);
      post("diag.log", 0.0);
      ++sl.dlog_count;
    }
  }
  int diag_log_read(int id, double* out, int maxrows) override {
    if (!dlog_every_) throw Error(LESGO_ERR_ARG, "diag log: not configured");
    const int slot = slot_of(id);
    const Slot& sl = slots_[slot];
    const int n = (int)std::min<long long>(sl.dlog_count, dlog_cap_);
    const int m = std::min(n, maxrows);
    std::vector<double> all((size_t)dlog_cap_ * 6);
    CK(cudaMemcpyAsync(all.data(), dlog_ + (long long)slot * dlog_cap_ * 6, all.size() * sizeof(double),
                       cudaMemcpyDeviceToHost, st_));
    CK(cudaStreamSynchronize(st_));
    // oldest first: the ring's first row is count % cap once it has wrapped
    const long long first = sl.dlog_count > dlog_cap_ ? sl.dlog_count % dlog_cap_ : 0;
    for (int r = 0; r < m; ++r) {
      const long long src = (first + (n - m) + r) % dlog_cap_;
      std::memcpy(out + 6 * r, all.data() + 6 * src, 6 * sizeof(double));
    }
    return m;
  }

  void counters(int id, int* jt, int* jt_total) const override {
    const Slot& sl = slots_[slot_of(id)];
    if (jt) *jt = sl.jt;
    if (jt_total) *jt_total = sl.jt_total;
  }

  void turbine_state(int id, double* udT, double* fn, double* pw, int n) override {
    const int slot = slot_of(id);
    int first = 0;
    for (int s = 0; s < slot; ++s) first += (int)slots_[s].spec.turbines.size();
    const int nt = (int)slots_[slot].spec.turbines.size();
    const int m = std::min(n, nt);
    std::vector<double> a(std::max(th_.n, 1)), b(std::max(th_.n, 1));
    if (th_.n) {
      CK(cudaStreamSynchronize(st_));
      CK(cudaMemcpy(a.data(), td_.u_d_T, th_.n * sizeof(double), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(b.data(), td_.f_n, th_.n * sizeof(double), cudaMemcpyDeviceToHost));
    }
    for (int s = 0; s < m; ++s) {
      if (udT) udT[s] = a[first + s];
      if (fn) fn[s] = b[first + s];
      if (pw) pw[s] = -b[first + s] * a[first + s];
    }
  }

  void turbine_schedule(int id, int which, int nt, const double* rows) override {
    const int slot = slot_of(id);
    InstanceSpec& sp = slots_[slot].spec;
    const int nloc = (int)sp.turbines.size();
    if (which < 0 || which > 2 || nt < 0 || (nt > 0 && !rows)) throw Error(LESGO_ERR_ARG, "bad schedule");
    if (nloc == 0) throw Error(LESGO_ERR_ARG, "instance has no turbines");
    std::vector<double> v(rows, rows + (size_t)nt * (1 + nloc));
    for (int r = 1; r < nt; ++r)
      if (!(v[(size_t)r * (1 + nloc)] >= v[(size_t)(r - 1) * (1 + nloc)]))
        throw Error(LESGO_ERR_ARG, "schedule times must not decrease");
    for (double x : v)
      if (!std::isfinite(x)) throw Error(LESGO_ERR_ARG, "schedule values must be finite");
    sp.sched[which] = v;
    rebuild_turbines(-1, -1);
    CK(cudaStreamSynchronize(st_));
  }
  void turbine_controls(int id, double* th1, double* th2, double* ctp, int n) override {
    const int slot = slot_of(id);
    const int first = turb_base_.count(slots_[slot].id) ? turb_base_[slots_[slot].id] : 0;
    const int m = std::min(n, (int)slots_[slot].spec.turbines.size());
    if (m <= 0 || !th_.n) return;
    std::vector<double> t(2 * th_.n), c(th_.n);
    CK(cudaStreamSynchronize(st_));
    CK(cudaMemcpy(t.data(), tctl_.theta, t.size() * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(c.data(), td_.ctp, c.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int s = 0; s < m; ++s) {
      if (th1) th1[s] = t[first + s];
      if (th2) th2[s] = t[th_.n + first + s];
      if (ctp) ctp[s] = c[first + s];
    }
  }

  int launches_per_step(int with_sgs) const override {
    auto it = launch_count_.find(with_sgs ? 1 : 0);
    return it == launch_count_.end() ? -1 : it->second;
  }

  // Profiling: eager steps with an event pair per launch; the report is a
  // JSON object {name: [launches, total_ms, total_bytes]}.
  void profile(int enable) override {
    CK(cudaStreamSynchronize(st_));
    for (auto& r : prof_) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    prof_.clear();
    prof_on_ = enable != 0;
    use_graphs_ = graphs_allowed_ && !prof_on_;
  }
  std::string profile_report() override {
    CK(cudaStreamSynchronize(st_));
    std::map<std::string, std::tuple<long long, double, double>> agg;
    for (auto& r : prof_) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, r.a, r.b));
      auto& t = agg[r.name];
      std::get<0>(t) += 1;
      std::get<1>(t) += ms;
      std::get<2>(t) += r.bytes;
    }
    std::string out = "{";
    bool first = true;
    for (auto& kv : agg) {
      char buf[512];
      std::snprintf(buf, sizeof(buf), "%s\"%s\": [%lld, %.6f, %.1f]", first ? "" : ", ", kv.first.c_str(),
                    std::get<0>(kv.second), std::get<1>(kv.second), std::get<2>(kv.second));
      out += buf;
      first = false;
    }
    return out + "}";
  }
  void* stream() const override { return (void*)st_; }

  // Stand-alone tridag_array on caller device arrays; the gam scratch is
  // owned by the handle and grows on demand.
  int tridag(const double* a, const double* b, const double* c, const double* r, double* u, int lh, int ny,
             int n) override {
    const long long need = (long long)lh * ny * n;
    if (need > tri_gam_n_) {
      if (tri_gam_) cudaFree(tri_gam_);
      tri_gam_ = nullptr;
      CK(cudaMalloc(&tri_gam_, need * sizeof(double)));
      tri_gam_n_ = need;
    }
    CK(cudaMemsetAsync(err_, 0, sizeof(int), st_));
    const int ncol = (lh - 1) * ny;
    pre();
    k_tridag<<<(ncol + 127) / 128, 128, 0, st_>>>(a, b, c, (const double2*)r, (double2*)u, tri_gam_, lh, ny, n, err_);
    post("tridag_array", (double)need * (3 * 8 + 2 * 16));
    int e = 0;
    CK(cudaMemcpyAsync(&e, err_, sizeof(int), cudaMemcpyDeviceToHost, st_));
    CK(cudaStreamSynchronize(st_));
    if (e) { CK(cudaMemset(err_, 0, sizeof(int))); return LESGO_ERR_NUMERIC; }
    return LESGO_OK;
  }

 private:
  struct Slot {
    int id = -1;
    InstanceSpec spec;
    int jt = 0, jt_total = 0;
    bool flm_init = false, fqn_init = false;
    int pending = 0;   // IF_INITLM / IF_INITQN set this step (committed after it)
    bool ta_init = false;          // time averaging started (tavg%init done)
    bool ta_loaded = false;        // sums read from tavg.out, taken up at the first sample
    bool initu = false;            // state read from a checkpoint of this grid (initial.f90:77-84)
    bool lag_prev = false;         // the previous step ran the dynamic update
    int flags = 0;                 // IF_* of the current step
    long long dlog_count = 0;      // rows written to the diagnostics log
  };

  int slot_of(int id) const {
    for (int s = 0; s < (int)slots_.size(); ++s)
      if (slots_[s].id == id) return s;
    throw Error(LESGO_ERR_ARG, "unknown instance id " + std::to_string(id));
  }
  void need_active() const {
    if (slots_.empty()) throw Error(LESGO_ERR_ARG, "no active instance");
  }
  InstMap imf(int nli) const { return InstMap(nli, kp_.istride); }

  void sync_instance_params() {
    kp_.ninst = (int)slots_.size();
    std::vector<double> zo(cap_, d_.p.zo);
    for (size_t s = 0; s < slots_.size(); ++s) zo[s] = slots_[s].spec.zo;
    CK(cudaMemcpyAsync(zo_d_, zo.data(), cap_ * sizeof(double), cudaMemcpyHostToDevice, st_));
    CK(cudaStreamSynchronize(st_));
  }

  // Copy a small int array to the device in stream order without waiting
  // for the stream: through the next slot of a pinned ring, reused only once
  // the copy that last read it has run (the host runs at most kRing uploads
  // ahead of the device).
  void upload_ints(int* dev, const std::vector<int>& v) {
    const int slot = (int)(ring_next_ % kRing);
    if (ring_next_ >= kRing) CK(cudaEventSynchronize(ring_ev_[slot]));
    int* h = ring_h_ + (size_t)slot * cap_;
    std::memcpy(h, v.data(), v.size() * sizeof(int));
    CK(cudaMemcpyAsync(dev, h, v.size() * sizeof(int), cudaMemcpyHostToDevice, st_));
    CK(cudaEventRecord(ring_ev_[slot], st_));
    ++ring_next_;
  }

  // Advance every instance's counters by one step and set its flags for the
  // step (main.f90:146-147, sgs_stag_util.f90:72-217, io.f90:557-562).
  void advance_counters() {
    for (auto& sl : slots_) {
      ++sl.jt;
      ++sl.jt_total;
      const bool inilag = !sl.initu;
      int f = 0;
      if (sl.jt_total == 1 && !sl.initu) f |= IF_EULER;
      const bool cs_fill = (sl.jt == 1 && inilag);
      if (cs_fill) f |= IF_CSFILL;
      if (!cs_fill && (sl.jt >= d_.p.dyn_init || sl.initu) && (sl.jt_total % d_.p.cs_count == 0)) {
        f |= IF_LAG;
        if (inilag && !sl.flm_init && (sl.jt == d_.p.cs_count || sl.jt == d_.p.dyn_init)) f |= IF_INITLM;
        if (inilag && !sl.fqn_init && (sl.jt == d_.p.cs_count || sl.jt == d_.p.dyn_init)) f |= IF_INITQN;
      }
      if (d_.p.use_cfl_dt) {
        if (sl.lag_prev) f |= IF_LAGRESET;
        if (sl.jt >= d_.p.dyn_init - d_.p.cs_count + 1 || sl.initu) f |= IF_LAGACC;
      }
      if (tavg_on_ && sl.jt_total >= ta_nstart_ && sl.jt_total <= ta_nend_) f |= IF_TAACC;
      sl.lag_prev = (f & IF_LAG) != 0;
      sl.pending = f & (IF_INITLM | IF_INITQN);
      sl.flags = f;
    }
  }
  // Upload this step's flags.  Returns true when a flag changes the kernels
  // the step launches (a step that is not replayed).
  bool upload_flags(bool* lag_any) {
    std::vector<int> fl(slots_.size(), 0);
    bool special = false, lag = false;
    for (size_t s = 0; s < slots_.size(); ++s) {
      const int f = slots_[s].flags;
      if (f & IF_SPECIAL) special = true;
      if (f & IF_LAG) lag = true;
      fl[s] = f;
    }
    upload_ints(flags_d_, fl);
    *lag_any = lag;
    return special;
  }
  // cfl_util.f90:70-111 and main.f90:135-150 on the device: the new dt (with
  // use_cfl_dt), total_time and the pending time-average weight.
  void step_begin_kernels() {
    if (d_.p.use_cfl_dt) {
      const long long m = (long long)d_.nx * d_.ny * (d_.nz - 1);
      const int nb = (int)std::max<long long>(1, std::min<long long>((m + 2047) / 2048, 1024));
      pre();
      k_cfl_max<R><<<dim3(nb, kp_.ninst), 256, 0, st_>>>(F_[LESGO_U], F_[LESGO_V], F_[LESGO_W], kp_, cflmax_d_);
      post("step.cfl_max", 3.0 * m * kp_.ninst * sizeof(R));
    }
    StepBeginArgs a;
    a.sc = sc_d_; a.iflags = flags_d_; a.mx = cflmax_d_; a.ninst = kp_.ninst; a.cfl_mode = d_.p.use_cfl_dt ? 1 : 0;
    a.cfl = d_.p.cfl; a.dx = d_.dx; a.dy = d_.dy; a.dz = d_.dz; a.c1 = 1.0 / ((double)d_.nx * d_.ny);
    a.z_i = d_.p.z_i; a.u_star = d_.p.u_star; a.T_avg_dim = d_.p.T_avg_dim;
    pre();
    k_step_begin<<<(kp_.ninst + 63) / 64, 64, 0, st_>>>(a);
    post("step.begin", 0.0);
  }
  // Step constants of a fresh instance (fixed time step values; with
  // use_cfl_dt the first step replaces them).
  void init_step_constants(int slot) {
    std::vector<double> c(SC_N, 0.0);
    const double dt = d_.p.dt;
    c[SC_DT] = dt; c[SC_DTF] = dt;
    c[SC_T1] = d_.tadv1; c[SC_T2] = d_.tadv2;
    c[SC_LDT] = d_.p.use_cfl_dt ? 0.0 : d_.lagran_dt;
    c[SC_PS] = 1.0 / ((double)d_.nx * d_.ny) / d_.tadv1 / dt;
    const double dt_dim = dt * d_.p.z_i / d_.p.u_star;
    c[SC_EPS] = d_.p.T_avg_dim > 0 ? (dt_dim / d_.p.T_avg_dim) / (1. + dt_dim / d_.p.T_avg_dim) : 1.0;
    CK(cudaMemcpyAsync(sc_d_ + (long long)slot * SC_N, c.data(), SC_N * sizeof(double), cudaMemcpyHostToDevice, st_));
    CK(cudaStreamSynchronize(st_));
  }
  double read_sc(int slot, int which) {
    double v = 0.0;
    CK(cudaMemcpyAsync(&v, sc_d_ + (long long)slot * SC_N + which, sizeof(double), cudaMemcpyDeviceToHost, st_));
    CK(cudaStreamSynchronize(st_));
    return v;
  }
  void write_sc(int slot, int which, double v) {
    CK(cudaMemcpyAsync(sc_d_ + (long long)slot * SC_N + which, &v, sizeof(double), cudaMemcpyHostToDevice, st_));
    CK(cudaStreamSynchronize(st_));
  }
  void commit_lagrange_init() {
    for (auto& sl : slots_) {
      if (sl.pending & IF_INITLM) sl.flm_init = true;
      if (sl.pending & IF_INITQN) sl.fqn_init = true;
      sl.pending = 0;
    }
  }

  void ic_slot(int slot, uint64_t seed) {
    const long long n = kp_.istride;
    k_ic<R><<<grid1(n), 256, 0, st_>>>(F_[LESGO_U], F_[LESGO_V], F_[LESGO_W], kp_, seed, slot);
    post();
  }

  void rebuild_turbines(int moved_to, int moved_from) {
    // Nothing queued or captured may read the disk arrays replaced below:
    // both streams drain and the captured steps (which hold the arrays and
    // the disk counts as launch parameters) are dropped before they are freed.
    CK(cudaStreamSynchronize(st_));
    CK(cudaStreamSynchronize(st2_));
    graphs_clear();
    // carry the disk-velocity state (u_d_T) of surviving turbines across the rebuild
    std::vector<double> old(std::max(th_.n, 1), -1.0);
    if (th_.n) CK(cudaMemcpy(old.data(), td_.u_d_T, th_.n * sizeof(double), cudaMemcpyDeviceToHost));
    std::vector<std::vector<lesgo_turbine_t>> per;
    std::vector<Schedules> sched;
    for (auto& sl : slots_) { per.push_back(sl.spec.turbines); sched.push_back(sl.spec.sched); }
    std::vector<double> state;
    for (size_t s = 0; s < slots_.size(); ++s) {
      const int id = slots_[s].id;
      auto it = turb_base_.find(id);
      for (size_t t = 0; t < slots_[s].spec.turbines.size(); ++t)
        state.push_back(it != turb_base_.end() && it->second + (int)t < (int)old.size() && th_.n ? old[it->second + t] : -1.0);
    }
    th_ = turbines_build(d_, per, sched, kp_.istride, ind_cache_);
    turb_base_.clear();
    int base = 0;
    for (auto& sl : slots_) { turb_base_[sl.id] = base; base += (int)sl.spec.turbines.size(); }
    for (void* q : turb_allocs_) cudaFree(q);
    turb_allocs_.clear();
    td_ = TurbDev{};
    tctl_ = TurbDyn{};
    cols_ = nullptr;
    kp_.turbines = th_.n > 0 ? 1 : 0;
    if (!kp_.turbines) return;
    if (!fza_uv_) fza_uv_ = alloc<R>(nfield_);
    td_.nturb = th_.n;
    td_.node_off = tupload(th_.node_off);
    td_.node_q = tupload(th_.node_q);
    td_.node_ind = tupload(th_.node_ind);
    td_.win_turb = tupload(th_.win_turb);
    td_.win_q = tupload(th_.win_q);
    td_.win_ind = tupload(th_.win_ind);
    td_.nwin = (int)th_.win_q.size();
    double* nhat_d = tupload(th_.nhat);
    double* ctp_d = tupload(th_.ctp);
    double* corr_d = tupload(th_.corr);
    double* ind_d = const_cast<double*>(td_.node_ind);
    td_.nhat = nhat_d; td_.ctp = ctp_d; td_.corr = corr_d;
    tctl_ = TurbDyn{};
    tctl_.nturb = th_.n; tctl_.adm = d_.p.adm_correction ? 1 : 0; tctl_.dyn_nodes = th_.dyn_nodes ? 1 : 0;
    tctl_.s_nt = tupload(th_.s_nt); tctl_.s_off = tupload(th_.s_off);
    tctl_.s_t = tupload(th_.s_t); tctl_.s_v = tupload(th_.s_v);
    tctl_.M = tupload(th_.Mv);
    tctl_.nhat = nhat_d; tctl_.ctp = ctp_d; tctl_.corr = corr_d;
    tctl_.theta = tupload(th_.theta);
    tctl_.sc = sc_d_;
    if (th_.dyn_nodes) {
      tctl_.dyn_list = tupload(th_.dyn_list);
      tctl_.ndyn = (int)th_.dyn_list.size();
      tctl_.node_off = td_.node_off;
      tctl_.box_r = tupload(th_.box_r);
      tctl_.node_ind = ind_d;
      tctl_.node_turb = tupload(th_.node_turb);
      tctl_.tab_off = tupload(th_.tab_off);
      tctl_.tab_r = tupload(th_.tab_r);
      tctl_.tab_R2 = tupload(th_.tab_R2);
      tctl_.tab_n = th_.tab_n;
      tctl_.ipar = tupload(th_.ipar);
      tctl_.cutoff = d_.p.filter_cutoff;
      tctl_.dx = d_.dx; tctl_.dy = d_.dy; tctl_.dz = d_.dz;
      tctl_.win_q = td_.win_q;
      tctl_.win_coff = tupload(th_.win_coff);
      tctl_.win_cand = tupload(th_.win_cand);
      tctl_.nwin = (int)th_.win_q.size();
    }
    td_.dia = tupload(th_.dia);
    td_.u_d = talloc<double>(th_.n);
    td_.u_d_T = tupload(state);
    td_.f_n = talloc<double>(th_.n);
    td_.disk = talloc<double>(th_.n);
    td_.tinst = tupload(th_.tinst);
    td_.sc = sc_d_;
    tctl_.tinst = td_.tinst;
    td_.dvol = d_.dx * d_.dy * d_.dz;
    cols_ = tupload(th_.cols);
    // the applied-force fields are rewritten only on disk nodes: clear them
    for (int f : {LESGO_FXA, LESGO_FYA, LESGO_FZA})
      CK(cudaMemsetAsync(F_[f], 0, nfield_ * sizeof(R), st_));
    CK(cudaMemsetAsync(fza_uv_, 0, nfield_ * sizeof(R), st_));
    CK(cudaStreamSynchronize(st_));
    (void)moved_to; (void)moved_from;
  }
  // Device arrays of the disks, freed at the next rebuild.
  template <typename T>
  T* talloc(long long n) {
    void* p = nullptr;
    CK(cudaMalloc(&p, std::max<long long>(n, 1) * sizeof(T)));
    turb_allocs_.push_back(p);
    CK(cudaMemsetAsync(p, 0, std::max<long long>(n, 1) * sizeof(T), st_));
    return (T*)p;
  }
  template <typename T>
  T* tupload(const std::vector<T>& v) {
    T* p = talloc<T>((long long)v.size());
    if (!v.empty()) CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st_));
    return p;
  }
  void graphs_clear() {
    for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
    graphs_.clear();
  }

  void step_body(bool lag_any) {
    step_begin_kernels();
    // main.f90:155-172: derivatives (RHS_f is saved inside the fused convec epilogue)
    const InstMap im = imf(d_.nz);
    SrcFields<R, 3> src{{F_[LESGO_U], F_[LESGO_V], F_[LESGO_W]}, (R)(1.0 / ((double)d_.nx * d_.ny)), 1, 1, d_.ld,
                        kp_.plane, im};
    // into the convective term's spectra, which reuses them (convec_part1)
    xfwd<3>(src, d_.nx, d_.ny, d_.nz, cvA_, px_, "filt_da.xfwd");
    ypass_lin<1, 3, true, true, T2, T2>(cvA_, 0, 1, d_.nz, d_.ny, specB_, d_.ny, d_.nz, 3, ROW_SAME,
                                        {{MUL_ONE}, {MUL_IKX}, {MUL_IKY}}, "filt_da.ypass");
    DstFields<R, 9> dst{{F_[LESGO_U], F_[LESGO_DUDX], F_[LESGO_DUDY], F_[LESGO_V], F_[LESGO_DVDX], F_[LESGO_DVDY],
                         F_[LESGO_W], F_[LESGO_DWDX], F_[LESGO_DWDY]}, 1, 1, d_.ld, kp_.plane, im};
    xinv<9>(dst, specB_, d_.nx, d_.ny, d_.nz, px_, "filt_da.xinv");
    // Two branches from here.  Branch: the applied forcing (filtered velocity
    // of this step, main.f90:248-257), then, once the column pass is done,
    // the dynamic update and the stress divergence.  Main: the wall-model
    // inputs (main.f90:180-189), sgs_stag with ddz and the wall values fused
    // (main.f90:164-189), the convective term.  They meet before the RHS
    // epilogue, which reads all of them.
    fork(0);
    if (kp_.turbines) on_branch([&] { turb_impl(); });
    wall_planes();
    if (!lag_any) column<COL_DDZ | COL_TAU>();
    else column<COL_DDZ | COL_STORE_S>();
    fork(1);
    on_branch([&] {
      if (lag_any) {
        lagrange();
        column<COL_READ_S | COL_TAU>();
      }
      divstress(3);
    });
    convec_part1(true);
    join(2);
    convec_part2(true);
    pressure_impl(true);
  }

  // ---------------- building blocks ----------------------------------------
  template <typename T>
  T* alloc(long long n) {
    void* p = nullptr;
    CK(cudaMalloc(&p, std::max<long long>(n, 1) * sizeof(T)));
    CK(cudaMemsetAsync(p, 0, std::max<long long>(n, 1) * sizeof(T), st_));
    allocs_.push_back(p);
    return (T*)p;
  }
  // Free one allocation of alloc() (the caller makes sure no queued work uses it).
  void release(void* p) {
    auto it = std::find(allocs_.begin(), allocs_.end(), p);
    if (it == allocs_.end()) return;
    cudaFree(*it);
    allocs_.erase(it);
  }
  double* staging(long long n) {
    if (n > staging_n_) {
      staging_ = alloc<double>(kp_.istride);
      staging_n_ = kp_.istride;
    }
    return staging_;
  }
  static dim3 grid1(long long n) { return dim3((unsigned)((n + 255) / 256)); }
  // Every launch is bracketed by pre() / post(name, bytes).  With profiling
  // on (eager steps only) an event pair on the handle's stream times it;
  // `bytes` is the launch's algorithmic traffic (unique inputs + outputs at
  // storage precision).
  void pre() {
    if (prof_on_) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e));
      CK(cudaEventRecord(e, st_));
      prof_start_ = e;
    }
  }
  void post(const char* name = "aux", double bytes = 0.0) {
    ++launches_;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error(LESGO_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    if (prof_on_ && prof_start_) {
      cudaEvent_t e1;
      CK(cudaEventCreate(&e1));
      CK(cudaEventRecord(e1, st_));
      prof_.push_back(ProfRec{name, bytes, prof_start_, e1});
      prof_start_ = nullptr;
    }
  }
  struct ProfRec { std::string name; double bytes; cudaEvent_t a, b; };
  template <typename KF>
  static void set_smem(KF kern, size_t bytes) {
    if (bytes > 48 * 1024) raise_smem_limit(reinterpret_cast<const void*>(kern), bytes);
  }

  FftPlan<A> make_plan(int n) {
    FftPlan<A> p{};
    p.n = n;
    auto r = factorize(n, !std::is_same<A, df64>::value);
    p.nf = (int)r.size();
    int ns = 1;
    for (int i = 0; i < p.nf; ++i) {
      p.radix[i] = r[i];
      p.nbs[i] = n / r[i];
      p.nss[i] = ns;
      p.fnb[i] = FastDiv((unsigned)p.nbs[i]);
      p.fns[i] = FastDiv((unsigned)ns);
      ns *= r[i];
    }
    std::vector<T2> tw(n), rtw(n + 1);
    for (int t = 0; t < n; ++t) {
      const long double a = -2.0L * kPiL * (long double)t / (long double)n;
      tw[t] = mkc(HostCvt<A>::from(cosl(a)), HostCvt<A>::from(sinl(a)));
    }
    for (int k = 0; k <= n; ++k) {
      const long double a = -2.0L * kPiL * (long double)k / (long double)(2 * n);
      rtw[k] = mkc(HostCvt<A>::from(cosl(a)), HostCvt<A>::from(sinl(a)));
    }
    // stage tables: butterfly jm's twiddles tw[r * jm * tws], r = 1..radix-1, side by side
    std::vector<T2> stw;
    for (int s = 0; s < p.nf; ++s) {
      p.two[s] = (int)stw.size();
      const int tws = p.nbs[s] / p.nss[s];
      if (s == 0) continue;
      for (int jm = 0; jm < p.nss[s]; ++jm)
        for (int r = 1; r < p.radix[s]; ++r) stw.push_back(tw[(size_t)r * jm * tws]);
    }
    T2* dtw = alloc<T2>(n);
    T2* drtw = alloc<T2>(n + 1);
    T2* dstw = alloc<T2>((long long)stw.size());
    CK(cudaMemcpyAsync(dtw, tw.data(), n * sizeof(T2), cudaMemcpyHostToDevice, st_));
    CK(cudaMemcpyAsync(drtw, rtw.data(), (n + 1) * sizeof(T2), cudaMemcpyHostToDevice, st_));
    if (!stw.empty()) CK(cudaMemcpyAsync(dstw, stw.data(), stw.size() * sizeof(T2), cudaMemcpyHostToDevice, st_));
    CK(cudaStreamSynchronize(st_));
    p.tw = dtw;
    p.rtw = drtw;
    p.stw = dstw;
    return p;
  }

  // Thomas pivots of every (kx, ky) column (tridag_array.f90:166-246): they
  // depend only on the wavenumbers and dz, so they are formed once in FP64.
  void build_thomas_pivots() {
    const int ny = d_.ny, K = d_.K, nz = d_.nz, n = nz + 1;
    const long long P = (long long)ny * K;
    std::vector<double> ib((size_t)(n + 1) * P, 1.0), gm((size_t)(n + 1) * P, 0.0);
    const double c3 = 1.0 / (d_.dz * d_.dz);
    for (int jy = 0; jy < ny; ++jy) {
      if (jy == ny / 2) continue;
      const int m = ((jy + ny / 2) % ny) - ny / 2;
      const double kyv = 2.0 * kPi / d_.p.L_y * (double)m;
      for (int jx = 0; jx < K; ++jx) {
        if (jx == 0 && jy == 0) continue;
        const double kxv = 2.0 * kPi / d_.p.L_x * (double)jx;
        const long long t = (long long)jy * K + jx;
        volatile double k2 = kxv * kxv;
        k2 = k2 + kyv * kyv;
        const double bmid = -(k2 + 2.0 * c3);
        double bet = -1.0;
        ib[P + t] = 1.0 / bet;
        for (int j = 2; j <= n; ++j) {
          const double cprev = (j == 2) ? 1.0 : c3;
          const double aj = (j <= nz) ? c3 : -1.0;
          const double bj = (j <= nz) ? bmid : 1.0;
          const double g = cprev / bet;
          bet = bj - aj * g;
          if (bet == 0.0) throw Error(LESGO_ERR_NUMERIC, "tridag_array: zero pivot");
          gm[(size_t)j * P + t] = g;
          ib[(size_t)j * P + t] = 1.0 / bet;
        }
      }
    }
    ibet_ = upload_vec(ib);
    tgam_ = upload_vec(gm);
  }

  void build_tables() {
    px_ = make_plan(d_.nx / 2);
    py_ = make_plan(d_.ny);
    pxb_ = make_plan(d_.nx2 / 2);
    pyb_ = make_plan(d_.ny2);
    // wavenumbers (fft.f90:130-160) for kx < nx/2 and every ky row
    const int ny = d_.ny, lh = d_.lh;
    std::vector<double> kx(d_.K), ky(ny);
    for (int jx = 0; jx < d_.K; ++jx) kx[jx] = 2.0 * kPi / d_.p.L_x * (double)jx;
    for (int jy = 0; jy < ny; ++jy) {
      const int m = ((jy + ny / 2) % ny) - ny / 2;
      ky[jy] = (jy == ny / 2) ? 0.0 : 2.0 * kPi / d_.p.L_y * (double)m;
    }
    // test-filter kernels (test_filtermodule.f90:38-123), (ny, lh)
    std::vector<double> G1((size_t)ny * lh), G2((size_t)ny * lh);
    for (int jy = 0; jy < ny; ++jy)
      for (int jx = 0; jx < lh; ++jx) {
        double kxv = (jx < lh - 1 && jy != ny / 2) ? 2.0 * kPi / d_.p.L_x * (double)jx : 0.0;
        const int m = ((jy + ny / 2) % ny) - ny / 2;
        double kyv = (jx < lh - 1 && jy != ny / 2) ? 2.0 * kPi / d_.p.L_y * (double)m : 0.0;
        volatile double k2 = kxv * kxv;
        k2 = k2 + kyv * kyv;
        for (int f = 0; f < 2; ++f) {
          const double alpha = f == 0 ? 2.0 : 4.0;
          const double dtest = alpha * std::sqrt(d_.dx * d_.dy);
          const double kc2 = (kPi / dtest) * (kPi / dtest);
          double g = 1.0 / ((double)d_.nx * d_.ny);
          if (k2 >= kc2) g = 0.0;
          if (jx == lh - 1 || jy == ny / 2) g = 0.0;
          (f == 0 ? G1 : G2)[(size_t)jy * lh + jx] = g;
        }
      }
    kxw_ = upload_as<A>(kx);
    kyw_ = upload_as<A>(ky);
    kxw64_ = upload_as<double>(kx);
    kyw64_ = upload_as<double>(ky);
    G1_ = upload_as<A>(G1);
    G2_ = upload_as<A>(G2);
    // the test filters vanish on every column past the cutoff circle: the y
    // pass writes zeros there without transforming
    for (int f = 0; f < 2; ++f) {
      const std::vector<double>& G = f == 0 ? G1 : G2;
      kmax_g_[f] = -1;
      for (int jy = 0; jy < ny; ++jy)
        for (int jx = 0; jx < lh; ++jx)
          if (G[(size_t)jy * lh + jx] != 0.0) kmax_g_[f] = std::max(kmax_g_[f], jx);
    }
  }
  template <typename T>
  T* upload_as(const std::vector<double>& v) {
    std::vector<T> t;
    t.reserve(v.size());
    for (double x : v) t.push_back(HostCvt<T>::from(x));
    T* p = alloc<T>((long long)t.size());
    CK(cudaMemcpyAsync(p, t.data(), t.size() * sizeof(T), cudaMemcpyHostToDevice, st_));
    CK(cudaStreamSynchronize(st_));
    return p;
  }
  template <typename T>
  T* upload_vec(const std::vector<T>& v) {
    T* p = alloc<T>((long long)v.size());
    if (!v.empty()) CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st_));
    CK(cudaStreamSynchronize(st_));
    return p;
  }

  // Batched passes over nli levels of every active instance.  Spectral
  // buffers hold [field][instance*nli + level][row][kx].
  template <int NF, class Src>
  void xfwd(const Src& src, int M, int nyrows, int nli, T2* out, const FftPlan<A>& plan, const char* tag = "xfwd",
            int in_fields = NF) {
    if constexpr (std::is_same<T2, float2>::value && std::is_same<typename Src::C, float2>::value) {
      if (xdft_w_ && M == d_.nx) {
        xfwd_tc<NF>(src, M, nyrows, nli, out, tag, in_fields);
        return;
      }
    }
    XfGeom g;
    g.M = M; g.K = d_.K; g.nyrows = nyrows; g.nrows = nyrows * nli * kp_.ninst; g.ls = M / 2 + 1;
    const int target = xtarget_;
    g.rpc = std::max(1, std::min(32, target / (NF * (M / 2))));
    g.out_field_stride = (long long)g.nrows * g.K;
    g.fH = FastDiv((unsigned)(M / 2)); g.fK = FastDiv((unsigned)g.K);
    g.fnyrows = FastDiv((unsigned)nyrows); g.frpc = FastDiv((unsigned)g.rpc);
    g.fnl = FastDiv((unsigned)(NF * g.rpc));
    const size_t smem = 2ull * NF * g.rpc * g.ls * sizeof(T2);
    auto kern = k_xfwd<A, NF, Src>;
    set_smem(kern, smem);
    pre();
    kern<<<(g.nrows + g.rpc - 1) / g.rpc, 256, smem, st_>>>(g, plan, src, out);
    post(tag, (double)g.nrows * ((double)in_fields * M * sizeof(R) + (double)NF * g.K * sizeof(T2)));
  }

  // The same transform as a tensor-core GEMM (k_xdft_tc): tiles of 128 rows,
  // one persistent block per SM (its shared memory holds W).
  template <int NF, class Src>
  void xfwd_tc(const Src& src, int M, int nyrows, int nli, float2* out, const char* tag, int in_fields) {
    XdGeom g{};
    g.M = M; g.K = d_.K; g.nyrows = nyrows; g.nrows = nyrows * nli * kp_.ninst;
    g.rpc = 128 / NF;
    g.ntiles = (g.nrows + g.rpc - 1) / g.rpc;
    g.pcols = (unsigned)((M + 31) / 32 * 32);
    g.ncols = 4 * g.pcols <= 128 ? 128u : 4 * g.pcols <= 256 ? 256u : 512u;
    g.out_field_stride = (long long)g.nrows * g.K;
    g.fnyrows = FastDiv((unsigned)nyrows);
    g.err = err_ + 1;
    // Blocks that share an SM must never ask for more than its 512
    // tensor-memory columns (an allocation would wait): enough shared
    // memory per block keeps their number at 512 / ncols or fewer.
    const size_t smem = std::max<size_t>(xdft_smem(M), g.ncols == 512 ? 116 * 1024 : g.ncols == 256 ? 78 * 1024 : 58 * 1024);
    if (smem > 227 * 1024) throw Error(LESGO_ERR_UNSUPPORTED, "x transform GEMM: shared memory");
    auto kern = k_xdft_tc<NF, Src>;
    set_smem(kern, smem);
    int nsm = 0, dev = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int grid = std::min(g.ntiles, nsm);
    pre();
    kern<<<grid, kXdThreads, smem, st_>>>(g, xdft_w_, src, out);
    post(tag, (double)g.nrows * ((double)in_fields * M * sizeof(R) + (double)NF * g.K * sizeof(T2)));
  }

  // kz_even / kz_odd: modes kx from which the even / odd input fields are
  // known to be zero (not read); -1: all K modes are read
  template <int NF, class Dst>
  void xinv(const Dst& dst, const T2* in, int M, int nyrows, int nli, const FftPlan<A>& plan, const char* tag = "xinv",
            int out_fields = NF, int kz_even = -1, int kz_odd = -1) {
    XiGeom g;
    g.M = M; g.K = d_.K; g.nyrows = nyrows; g.nrows = nyrows * nli * kp_.ninst; g.ls = M / 2 + 1;
    g.kz0 = kz_even < 0 ? g.K : std::min(kz_even, g.K);
    g.kz1 = kz_odd < 0 ? g.K : std::min(kz_odd, g.K);
    const int target = xtarget_;
    g.rpc = std::max(1, std::min(32, target / (NF * (M / 2))));
    g.in_field_stride = (long long)g.nrows * g.K;
    g.fH = FastDiv((unsigned)(M / 2)); g.fM = FastDiv((unsigned)M);
    g.fnyrows = FastDiv((unsigned)nyrows); g.frpc = FastDiv((unsigned)g.rpc);
    g.fnl = FastDiv((unsigned)(NF * g.rpc));
    const size_t smem = 2ull * NF * g.rpc * g.ls * sizeof(T2);
    auto kern = k_xinv<A, NF, Dst>;
    set_smem(kern, smem);
    pre();
    kern<<<(g.nrows + g.rpc - 1) / g.rpc, 256, smem, st_>>>(g, plan, in, dst);
    post(tag, (double)g.nrows * ((double)NF * g.K * sizeof(T2) + (double)out_fields * M * sizeof(R)));
  }

  // Y pass over groups of NIN inputs -> NOUT outputs, nli levels of every
  // instance.  Input field g*NIN+i holds in_inst_levels planes per instance
  // (read at in_lev0 + level*in_levstride); outputs are contiguous.
  template <int NIN, int NOUT, bool FWD, bool INV, typename InT, typename OutT>
  void ypass_lin(const InT* in, int in_lev0, int in_levstride, int in_inst_levels, int in_rows, OutT* out,
                 int out_rows, int nli, int ngroups, int rowmode, std::initializer_list<std::initializer_list<int>> mul,
                 const char* tag = "ypass", bool store_zero_tiles = true) {
    const int nlev = nli * kp_.ninst;
    YOpLin<A, NIN, NOUT, InT, OutT> op;
    op.in = in;
    op.in_fs = (long long)in_inst_levels * kp_.ninst * in_rows * d_.K;
    op.in_lev0 = in_lev0; op.in_levstride = in_levstride; op.in_rows = in_rows;
    op.nli = nli; op.in_inst_levels = in_inst_levels; op.fnli = FastDiv((unsigned)nli);
    op.out = out; op.out_fs = (long long)nlev * out_rows * d_.K; op.out_rows = out_rows;
    op.K = d_.K; op.lh = d_.lh; op.ny_small = d_.ny; op.ny_big = d_.ny2; op.rowmode = rowmode;
    int o = 0;
    for (auto& row : mul) {
      int i = 0;
      for (int m : row) { if (o < NOUT && i < NIN) op.mul[o][i] = m; ++i; }
      for (; i < NIN; ++i) op.mul[o][i] = MUL_ZERO;
      ++o;
    }
    op.kxw = kxw_; op.kyw = kyw_; op.G1 = G1_; op.G2 = G2_;
    op.store_zero = store_zero_tiles || !yshort_;
    for (int o = 0; o < NOUT; ++o) {
      // zero from the first column past its test filters' cutoffs (or never)
      int zf = -1;
      bool kxonly = true;
      for (int i = 0; i < NIN; ++i) {
        const int m = op.mul[o][i];
        if (m == MUL_ZERO) continue;
        if (m != MUL_ONE && m != MUL_IKX) kxonly = false;
        if (m == MUL_G1 || m == MUL_G2) zf = std::max(zf, kmax_g_[m == MUL_G1 ? 0 : 1] + 1);
        else zf = 1 << 30;
      }
      op.zero_from[o] = zf < 0 ? 0 : zf;
      op.sc_out[o] = kxonly && zf >= 0;
      if (!yshort_) { op.zero_from[o] = 1 << 30; op.sc_out[o] = false; }
    }
    // inverse-only passes: an output that is i kx times an earlier output
    // (MUL_IKX where the earlier one has MUL_ONE, zero elsewhere) takes the
    // earlier output's inverse transform
    for (int o2 = 0; o2 < NOUT; ++o2) {
      op.from[o2] = -1;
      op.from_in[o2] = 0;
    }
    if constexpr (!FWD && INV) {
      for (int o2 = 0; o2 < NOUT && rowmode == ROW_SAME && yshort_; ++o2) {
        for (int o1 = 0; o1 < o2 && op.from[o2] < 0; ++o1) {
          bool match = true, any = false;
          int fin = 0;
          for (int i = 0; i < NIN; ++i) {
            const int a = op.mul[o1][i], b = op.mul[o2][i];
            if (a == MUL_ZERO && b == MUL_ZERO) continue;
            if (a == MUL_ONE && b == MUL_IKX) { any = true; fin = i; continue; }
            match = false;
          }
          if (match && any && op.from[o1] < 0) { op.from[o2] = o1; op.from_in[o2] = fin; }
        }
      }
    }
    YGeom g;
    g.ny_in = in_rows; g.ny_out = out_rows; g.K = d_.K; g.nlev = nlev;
    g.ls_in = in_rows + 1; g.ls_out = out_rows + 1;
    const FftPlan<A>& pin = (in_rows == d_.ny) ? py_ : pyb_;
    const FftPlan<A>& pout = (out_rows == d_.ny) ? py_ : pyb_;
    const size_t budget = ybudget_;
    int tk = sizeof(T2) == 16 ? 8 : 16;
    auto smem_of = [&](int t) {
      const size_t s = (size_t)NIN * t * g.ny_in;
      return (s + std::max(s, (size_t)2 * t * g.ny_out)) * sizeof(T2);
    };
    while (tk > 1 && smem_of(tk) > budget) tk /= 2;
    while (tk > d_.K) tk /= 2;          // tk stays a power of two
    while (tk > 1 && d_.K % tk != 0) tk /= 2;   // no partly empty tile (K = 24 -> 8 columns)
    g.tk = tk;
    g.tk_log2 = 0;
    while ((1 << g.tk_log2) < tk) ++g.tk_log2;
    g.fny_in = FastDiv((unsigned)in_rows); g.fny_out = FastDiv((unsigned)out_rows);
    g.fwin = FastDiv((unsigned)(NIN * tk));
    g.ftk = FastDiv((unsigned)tk);
    g.in_lev_stride = 0; g.out_lev_stride = 0;
    const size_t smem = smem_of(tk);
    dim3 grid((d_.K + tk - 1) / tk, nlev, ngroups);
    // an output whose operator depends on kx alone needs no y transform:
    // the instance with that path, for the one-input passes that have one
    bool sc = false;
    if constexpr (FWD && INV && NIN == 1) {
      if (rowmode == ROW_SAME && in_rows == out_rows)
        for (int o = 0; o < NOUT; ++o) sc |= op.sc_out[o];
      if (sc) {
        auto kern = k_ypass<A, NIN, NOUT, FWD, INV, true, YOpLin<A, NIN, NOUT, InT, OutT>>;
        set_smem(kern, smem);
        pre();
        kern<<<grid, ythreads_, smem, st_>>>(g, pin, pout, op);
      }
    }
    if (!sc) {
      auto kern = k_ypass<A, NIN, NOUT, FWD, INV, false, YOpLin<A, NIN, NOUT, InT, OutT>>;
      set_smem(kern, smem);
      pre();
      kern<<<grid, ythreads_, smem, st_>>>(g, pin, pout, op);
    }
    post(tag, (double)ngroups * nlev * d_.K *
                  ((double)NIN * in_rows * sizeof(InT) + (double)NOUT * out_rows * sizeof(OutT)));
  }

  // test filter (G_test) of plane `level` of two fields into two planes per
  // instance (out planes are `ostr` apart between instances)
  void filter_planes(const R* a, const R* b, int level, R* oa, R* ob, int nf, long long ostr) {
    const long long pl_s = (long long)d_.ny * d_.K;
    T2* in = specC_;
    T2* outp = specC_ + 2 * pl_s * kp_.ninst;
    SrcFields<R, 2> src{{a, b}, (R)1, level, 1, d_.ld, kp_.plane, imf(1)};
    xfwd<2>(src, d_.nx, d_.ny, 1, in, px_, "wall_filter.xfwd");
    ypass_lin<1, 1, true, true, T2, T2>(in, 0, 1, 1, d_.ny, outp, d_.ny, 1, 2, ROW_SAME, {{MUL_G1}}, "wall_filter.ypass");
    if (nf == 1) {
      DstFields<R, 1> dst{{oa}, 0, 1, d_.ld, 0, InstMap(1, ostr)};
      xinv<1>(dst, outp, d_.nx, d_.ny, 1, px_, "wall_filter.xinv");
    } else {
      DstFields<R, 2> dst{{oa, ob}, 0, 1, d_.ld, 0, InstMap(1, ostr)};
      xinv<2>(dst, outp, d_.nx, d_.ny, 1, px_, "wall_filter.xinv");
    }
  }
  void wall_planes() {
    if (d_.p.lbc_mom == 2) filter_planes(F_[LESGO_U], F_[LESGO_V], 1, wall_[0], wall_[1], 2, kp_.plane);
    if (d_.p.ubc_mom == 2) filter_planes(F_[LESGO_U], F_[LESGO_V], d_.nz - 1, wall_[2], wall_[3], 2, kp_.plane);
  }

  template <int FLAGS>
  void column() {
    ColArgs<R> a;
    a.u = F_[LESGO_U]; a.v = F_[LESGO_V]; a.w = F_[LESGO_W];
    a.dudx = F_[LESGO_DUDX]; a.dudy = F_[LESGO_DUDY]; a.dvdx = F_[LESGO_DVDX]; a.dvdy = F_[LESGO_DVDY];
    a.dwdx = F_[LESGO_DWDX]; a.dwdy = F_[LESGO_DWDY];
    a.dudz = F_[LESGO_DUDZ]; a.dvdz = F_[LESGO_DVDZ]; a.dwdz = F_[LESGO_DWDZ];
    a.S11 = F_[LESGO_S11]; a.S12 = F_[LESGO_S12]; a.S13 = F_[LESGO_S13];
    a.S22 = F_[LESGO_S22]; a.S23 = F_[LESGO_S23]; a.S33 = F_[LESGO_S33];
    a.Cs = F_[LESGO_CS_OPT2];
    a.txx = F_[LESGO_TXX]; a.txy = F_[LESGO_TXY]; a.txz = F_[LESGO_TXZ];
    a.tyy = F_[LESGO_TYY]; a.tyz = F_[LESGO_TYZ]; a.tzz = F_[LESGO_TZZ];
    a.wb_u = wall_[0]; a.wb_v = wall_[1]; a.wt_u = wall_[2]; a.wt_v = wall_[3];
    a.kp = kp_;
    a.delta2 = d_.delta * d_.delta;
    a.chunk = 16;
    const int ncol = d_.nx * d_.ny;
    dim3 grid((ncol + 255) / 256, (d_.nz + a.chunk - 1) / a.chunk, kp_.ninst);
    const int nrw = (FLAGS & COL_READ_S) ? 13 : (FLAGS & COL_TAU) ? 19 : 18;
    pre();
    k_column<R, FLAGS><<<grid, 256, 0, st_>>>(a);
    post((FLAGS & COL_READ_S) ? "sgs_column.tau" : (FLAGS & COL_TAU) ? "sgs_column" : "sgs_column.sij",
         (double)nrw * ncol * d_.nz * kp_.ninst * sizeof(R));
  }

  void lagrange() {
    InterpArgs<R> ia;
    ia.u = F_[LESGO_U]; ia.v = F_[LESGO_V]; ia.w = F_[LESGO_W];
    const int Fi[4] = {LESGO_F_LM, LESGO_F_MM, LESGO_F_QN, LESGO_F_NN};
    for (int f = 0; f < 4; ++f) { ia.Fin[f] = F_[Fi[f]]; ia.Fout[f] = Ftmp_[f]; }
    ia.kp = kp_;
    const long long n = (long long)d_.nx * d_.ny * d_.nz * kp_.ninst;
    pre();
    k_interp<R><<<grid1(n), 256, 0, st_>>>(ia);
    post("lagrange.interp", 11.0 * n * sizeof(R));
    SrcLagrange<R> src{F_[LESGO_U], F_[LESGO_V], F_[LESGO_W], F_[LESGO_S11], F_[LESGO_S12], F_[LESGO_S13],
                       F_[LESGO_S22], F_[LESGO_S23], F_[LESGO_S33], d_.ld, d_.nz, kp_.lbc, kp_.ubc, kp_.plane,
                       imf(d_.nz)};
    xfwd<21>(src, d_.nx, d_.ny, d_.nz, specA_, px_, "lagrange.xfwd", 9);
    // the 2-delta (even outputs) and 4-delta (odd) filtered spectra are zero
    // past the filters' cutoff columns: the y pass does not write those
    // tiles and the x inverse does not read those modes
    ypass_lin<1, 2, true, true, T2, T2>(specA_, 0, 1, d_.nz, d_.ny, specB_, d_.ny, d_.nz, 21, ROW_SAME,
                                        {{MUL_G1}, {MUL_G2}}, "lagrange.ypass", false);
    DstLagrange<R> dst;
    dst.FLMi = Ftmp_[0]; dst.FMMi = Ftmp_[1]; dst.FQNi = Ftmp_[2]; dst.FNNi = Ftmp_[3];
    dst.FLM = F_[LESGO_F_LM]; dst.FMM = F_[LESGO_F_MM]; dst.FQN = F_[LESGO_F_QN]; dst.FNN = F_[LESGO_F_NN];
    dst.Cs = F_[LESGO_CS_OPT2]; dst.Beta = F_[LESGO_BETA]; dst.Tn_all = F_[LESGO_TN_ALL]; dst.ee_now = F_[LESGO_EE_NOW];
    dst.cst = 2.0 * (d_.delta * d_.delta);
    dst.opftdelta = 1.5 * d_.delta;
    dst.sc = sc_d_;
    dst.beta_exp = std::log(2.0) / (std::log(4.0) - std::log(2.0));
    dst.beta_exp_one = dst.beta_exp == 1.0;
    dst.ld = d_.ld; dst.nz = d_.nz; dst.lbc = kp_.lbc; dst.ubc = kp_.ubc;
    dst.iflags = flags_d_;
    dst.plane = kp_.plane;
    dst.im = imf(d_.nz);
    xinv<42>(dst, specB_, d_.nx, d_.ny, d_.nz, px_, "lagrange.xinv", 13, kmax_g_[0] + 1, kmax_g_[1] + 1);
  }

  // convec.f90:21-333: vorticity and velocity to the 3/2 grid, the three
  // products there, back to the kept modes (part 1); the RHS epilogue, with
  // the AB2 advance when fused (part 2).
  void convec_impl(bool fused) {
    convec_part1(false);
    convec_part2(fused);
  }
  // uvw_ready: the first three spectra of cvA_ already hold the x transforms
  // of u, v, w (filt_da's forward pass in the fused step).  They are those of
  // the field before filt_da's filter, which differs from the filtered field
  // only in the ky = ny/2 row, and the 3/2 padding below drops that row.
  void convec_part1(bool uvw_ready) {
    const R c = (R)(1.0 / ((double)d_.nx * d_.ny));
    const InstMap im = imf(d_.nz);
    const InstMap imb(d_.nz, kp_.istride_big);
    if (uvw_ready) {
      SrcVort<R, true> sv{F_[LESGO_U], F_[LESGO_V], F_[LESGO_W], F_[LESGO_DUDY], F_[LESGO_DUDZ], F_[LESGO_DVDX],
                          F_[LESGO_DVDZ], F_[LESGO_DWDX], F_[LESGO_DWDY], c, d_.ld, d_.nz, kp_.lbc, kp_.ubc,
                          kp_.plane, im};
      xfwd<3>(sv, d_.nx, d_.ny, d_.nz, cvA_ + 3 * vol1_s_ * kp_.ninst, px_, "convec.xfwd", 6);
    } else {
      SrcVort<R> sv{F_[LESGO_U], F_[LESGO_V], F_[LESGO_W], F_[LESGO_DUDY], F_[LESGO_DUDZ], F_[LESGO_DVDX],
                    F_[LESGO_DVDZ], F_[LESGO_DWDX], F_[LESGO_DWDY], c, d_.ld, d_.nz, kp_.lbc, kp_.ubc, kp_.plane, im};
      xfwd<6>(sv, d_.nx, d_.ny, d_.nz, cvA_, px_, "convec.xfwd", 9);
    }
    ypass_lin<1, 1, true, true, T2, T2>(cvA_, 0, 1, d_.nz, d_.ny, cvB_, d_.ny2, d_.nz, 6, ROW_PAD, {{MUL_ONE}},
                                        "convec.ypass_pad");
    if (conv_rows_) {
      convec_rows(HostCvt<A>::from(1.0L / ((long double)d_.nx2 * d_.ny2)));
    } else {
      DstFields<R, 6> db{{big_[0], big_[1], big_[2], big_[3], big_[4], big_[5]}, 1, 1, d_.ld_big, kp_.plane_big, imb};
      xinv<6>(db, cvB_, d_.nx2, d_.ny2, d_.nz, pxb_, "convec.xinv_big");
      const R cb = (R)(1.0 / ((double)d_.nx2 * d_.ny2));
      SrcConvProd<R> sp{big_[0], big_[1], big_[2], big_[3], big_[4], big_[5], cb, d_.ld_big, d_.nz, kp_.plane_big,
                        imb};
      xfwd<3>(sp, d_.nx2, d_.ny2, d_.nz, cvA_, pxb_, "convec.xfwd_big", 6);
    }
    ypass_lin<1, 1, true, true, T2, T2>(cvA_, 0, 1, d_.nz, d_.ny2, cvB_, d_.ny, d_.nz, 3, ROW_UNPAD, {{MUL_ONE}},
                                        "convec.ypass_unpad");
  }
  // The 3/2-grid x-rows of the convective term in one pass: the six padded
  // spectra of cvB_ in, the three products' x-spectra (nx/2 modes) into cvA_.
  void convec_rows(A cb) {
    ConvRowsGeom g;
    g.M = d_.nx2; g.K = d_.K; g.ny2 = d_.ny2; g.nz = d_.nz; g.ls = d_.nx2 / 2 + 1;
    g.in_fs = vol1_b_ * kp_.ninst;
    g.out_fs = vol1_b_ * kp_.ninst;
    const int H = d_.nx2 / 2;
    // rows per block as for the other x passes, within a shared-memory
    // budget of three blocks per SM (two for 16-byte complex values): fewer
    // rows leave most threads idle in the radix-8 stages; one complex
    // element more holds the copy barrier
    int rt = std::max(1, std::min(16, xtarget_ / (6 * H)));
    auto smem_of = [&](int r) { return (size_t)(conv_rows_smem_elems(r, g.ls, d_.K) + 1) * sizeof(T2); };
    const size_t budget = (sizeof(T2) == 16 ? 112 : 74) * 1024;
    while (rt > 1 && smem_of(rt) > budget) --rt;
    g.rt = rt;
    g.fH = FastDiv((unsigned)H); g.fK = FastDiv((unsigned)d_.K);
    g.f2 = FastDiv((unsigned)(2 * rt)); g.f3 = FastDiv((unsigned)(3 * rt)); g.f6 = FastDiv((unsigned)(6 * rt));
    g.frt = FastDiv((unsigned)rt);
    g.err = err_ + 1;
    const size_t smem = smem_of(rt);
    auto kern = k_convec_rows<A>;
    set_smem(kern, smem);
    // Levels per chunk: every block marches its chunk (plus up to two
    // levels of halo), so the launch takes about (waves) x (chunk + 2)
    // level times, with waves = blocks / resident blocks.  The chunk count
    // that minimises it keeps the last wave full (at 128^3: 7 chunks of 19
    // levels, one wave, against 9 chunks of 16 levels in two).
    const long long tiles = (long long)((d_.ny2 + rt - 1) / rt) * kp_.ninst;
    int per_sm = 0, nsm = 0, dev = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem));
    const long long slots = std::max(1LL, (long long)per_sm * nsm);
    int best_n = 1;
    long long best_t = -1;
    for (int n = 1; n <= d_.nz; ++n) {
      const long long waves = (tiles * n + slots - 1) / slots;
      const long long t = waves * ((d_.nz + n - 1) / n + 2);
      if (best_t < 0 || t < best_t) { best_t = t; best_n = n; }
    }
    g.cz = (d_.nz + best_n - 1) / best_n;
    dim3 grid((unsigned)((d_.ny2 + rt - 1) / rt), (unsigned)((d_.nz + g.cz - 1) / g.cz), (unsigned)kp_.ninst);
    pre();
    kern<<<grid, 256, smem, st_>>>(g, pxb_, cvB_, cvA_, cb);
    post("convec.rows", 9.0 * vol1_b_ * kp_.ninst * sizeof(T2));
  }
  void convec_part2(bool fused) {
    const InstMap im = imf(d_.nz);
    if (!fused) {
      DstConvec<R, false> dc{};
      dc.RHSx = F_[LESGO_RHSX]; dc.RHSy = F_[LESGO_RHSY]; dc.RHSz = F_[LESGO_RHSZ];
      dc.ld = d_.ld; dc.nz = d_.nz; dc.plane = kp_.plane; dc.iflags = flags_d_; dc.im = im;
      xinv<3>(dc, cvB_, d_.nx, d_.ny, d_.nz, px_);
    } else {
      DstConvec<R, true> dc{};
      dc.RHSx = F_[LESGO_RHSX]; dc.RHSy = F_[LESGO_RHSY]; dc.RHSz = F_[LESGO_RHSZ];
      dc.RHSxf = F_[LESGO_RHSX_F]; dc.RHSyf = F_[LESGO_RHSY_F]; dc.RHSzf = F_[LESGO_RHSZ_F];
      dc.u = F_[LESGO_U]; dc.v = F_[LESGO_V]; dc.w = F_[LESGO_W];
      dc.divtx = F_[LESGO_DIVTX]; dc.divty = F_[LESGO_DIVTY]; dc.divtz = F_[LESGO_DIVTZ];
      dc.fxa = F_[LESGO_FXA]; dc.fya = F_[LESGO_FYA]; dc.fza = F_[LESGO_FZA];
      dc.sc = sc_d_; dc.mpfx = d_.mpfx; dc.mpfy = d_.mpfy;
      dc.ld = d_.ld; dc.nz = d_.nz; dc.use_mpf = d_.p.use_mean_p_force; dc.turbines = kp_.turbines;
      dc.iflags = flags_d_; dc.plane = kp_.plane; dc.im = im;
      xinv<3>(dc, cvB_, d_.nx, d_.ny, d_.nz, px_, "convec.xinv_ab2", 18 + 3 * kp_.turbines);
    }
  }

  // Fork: work launched between fork() and join() with on_branch = true runs
  // on the second stream once the main stream has reached the fork; join()
  // makes the main stream wait for the branch.  Both are graph-capturable.
  // While profiling (or with LESGO_BRANCHES=0, for external profilers),
  // branches run on the main stream, so that each kernel is timed alone.
  bool serial() const { return prof_on_ || !branches_allowed_; }
  void fork(int e) {
    if (serial()) return;
    CK(cudaEventRecord(ev_[e], st_));
    CK(cudaStreamWaitEvent(st2_, ev_[e], 0));
  }
  void join(int e) {
    if (serial()) return;
    CK(cudaEventRecord(ev_[e], st2_));
    CK(cudaStreamWaitEvent(st_, ev_[e], 0));
  }
  template <class F>
  void on_branch(F&& fn) {
    if (serial()) {
      fn();
      return;
    }
    std::swap(st_, st2_);
    try {
      fn();
    } catch (...) {
      std::swap(st_, st2_);
      throw;
    }
    std::swap(st_, st2_);
  }

  void pressure_impl(bool fused) {
    const int nz = d_.nz, ny = d_.ny;
    const long long pl_s = (long long)ny * d_.K;
    const double c1 = 1.0 / ((double)d_.nx * d_.ny);
    // scale 1/(nx ny tadv1 dt), the instance's step constant SC_PS
    SrcFields<R, 3> su{{F_[LESGO_U], F_[LESGO_V], F_[LESGO_W]}, (R)0, 1, 1, d_.ld, kp_.plane, imf(nz), sc_d_, SC_PS};
    xfwd<3>(su, d_.nx, ny, nz, specA_, px_, "press.xfwd");
    // the boundary planes (divtz at levels 1 and nz) on the second stream
    fork(3);
    on_branch([&] {
      SrcFields<R, 1> sd{{F_[LESGO_DIVTZ]}, (R)c1, 1, nz - 1, d_.ld, kp_.plane, imf(2)};
      xfwd<1>(sd, d_.nx, ny, 2, specC_, px_, "press.xfwd_bc");
      ypass_lin<1, 1, true, false, T2, double2>(specC_, 0, 1, 2, ny, hplane_, ny, 2, 1, ROW_SAME, {{MUL_ONE}},
                                                "press.ypass_fwd_bc");
    });
    ypass_lin<1, 1, true, false, T2, double2>(specA_, 0, 1, nz, ny, hspec_, ny, nz, 3, ROW_SAME, {{MUL_ONE}},
                                              "press.ypass_fwd");
    join(4);
    const long long vs = vol1_s_ * kp_.ninst;
    ThomasArgs ta;
    ta.Hx = hspec_; ta.Hy = hspec_ + vs; ta.Hz = hspec_ + 2 * vs;
    ta.Hb = hplane_; ta.Ht = hplane_ + pl_s;
    ta.phat = phat_; ta.ibet = ibet_; ta.gam = tgam_;
    ta.kxw = kxw64_; ta.kyw = kyw64_;
    ta.dz = d_.dz; ta.idz = 1.0 / d_.dz; ta.idz2 = 1.0 / (d_.dz * d_.dz);
    ta.nz = nz; ta.ny = ny; ta.K = d_.K; ta.ninst = kp_.ninst;
    pre();
    // The FP64 pipe bounds this solve on GB300.  With enough columns (a
    // batch; measured: 17280 columns 20 % and 45056 columns 51 % faster
    // than segmented) one thread sweeps each column in order, which does
    // half the FP64 work of the segmented forms; with fewer columns (one
    // 128^3 instance: 8320) the segmented forms keep the SMs busy: 16
    // segments held in registers up to 192 unknowns, the looped form beyond.
    // LESGO_THOMAS=seq|seg forces a form.
    const long long ncol = pl_s * kp_.ninst;
    const int nu = nz + 1;
    const bool seq = thomas_mode_ == 1 || (thomas_mode_ == 0 && ncol >= 12288);
    // four levels per register chunk: 96 registers a thread (164 with
    // eight), so the sweep leaves room on the SMs for the other handles'
    // kernels running beside it (the ensemble step measured 1 % shorter;
    // the sweep alone takes the same time)
    if (seq)
      k_thomas_seq<4><<<(unsigned)((ncol + 127) / 128), 128, 0, st_>>>(ta);
    else if (nu <= 192)
      k_thomas_r<16, 8, 12><<<(unsigned)((ncol + 7) / 8), 128, 0, st_>>>(ta);
    else
      k_thomas<16, 16><<<(unsigned)((ncol + 15) / 16), 256, 0, st_>>>(ta);
    post("press.thomas", (double)pl_s * kp_.ninst * (4.0 * nz + 1.0) * sizeof(double2));
    // p, i kx p, i ky p at levels 1..nz-1; p at levels 0 and nz (phat holds nz+1 planes per instance)
    // p at levels 0 and nz on the second stream
    fork(5);
    on_branch([&] {
      ypass_lin<1, 1, false, true, double2, T2>(phat_, 0, nz, nz + 1, ny, specC_, ny, 2, 1, ROW_SAME, {{MUL_ONE}},
                                                "press.ypass_inv_bc");
      DstFields<R, 1> d0{{F_[LESGO_P]}, 0, nz, d_.ld, kp_.plane, imf(2)};
      xinv<1>(d0, specC_, d_.nx, ny, 2, px_, "press.xinv_bc");
    });
    ypass_lin<1, 3, false, true, double2, T2>(phat_, 1, 1, nz + 1, ny, specB_, ny, nz - 1, 1, ROW_SAME,
                                              {{MUL_ONE}, {MUL_IKX}, {MUL_IKY}}, "press.ypass_inv");
    if (fused) {
      DstPress<R, true> dp{F_[LESGO_P], F_[LESGO_DPDX], F_[LESGO_DPDY], F_[LESGO_RHSX], F_[LESGO_RHSY], F_[LESGO_U],
                           F_[LESGO_V], sc_d_, d_.ld, kp_.plane, imf(nz - 1)};
      xinv<3>(dp, specB_, d_.nx, ny, nz - 1, px_, "press.xinv_project", 9);
    } else {
      DstPress<R, false> dp{F_[LESGO_P], F_[LESGO_DPDX], F_[LESGO_DPDY], F_[LESGO_RHSX], F_[LESGO_RHSY], F_[LESGO_U],
                            F_[LESGO_V], sc_d_, d_.ld, kp_.plane, imf(nz - 1)};
      xinv<3>(dp, specB_, d_.nx, ny, nz - 1, px_);
    }
    join(6);
    const long long n = (long long)d_.nx * ny * nz * kp_.ninst;
    pre();
    if (fused)
      k_wproj<R, true><<<grid1(n), 256, 0, st_>>>(F_[LESGO_P], F_[LESGO_DPDZ], F_[LESGO_RHSZ], F_[LESGO_U], F_[LESGO_V],
                                                  F_[LESGO_W], kp_);
    else
      k_wproj<R, false><<<grid1(n), 256, 0, st_>>>(F_[LESGO_P], F_[LESGO_DPDZ], F_[LESGO_RHSZ], F_[LESGO_U], F_[LESGO_V],
                                                   F_[LESGO_W], kp_);
    post("press.wproj", (fused ? 5.0 : 2.0) * n * sizeof(R));
  }

  void turb_impl() {
    if (th_.dyn_ctl) {
      pre();
      k_turb_controls<<<(th_.n + 63) / 64, 64, 0, st_>>>(tctl_);
      post("turbines.controls", 0.0);
    }
    if (th_.dyn_nodes && !th_.dyn_list.empty()) {
      pre();
      k_turb_nodes<<<(unsigned)th_.dyn_list.size(), 256, 0, st_>>>(tctl_);
      post("turbines.nodes", (double)th_.node_q.size() * 40.0);
    }
    pre();
    k_turb_disk<R><<<th_.n, 256, 0, st_>>>(td_, F_[LESGO_U], F_[LESGO_V], F_[LESGO_W], kp_.plane, d_.nz, kp_.istride);
    post("turbines.disk", (double)th_.node_q.size() * (4 * sizeof(R) + 16.0));
    if (td_.nwin > 0) {
      pre();
      if (th_.dyn_nodes)
        k_turb_scatter_dyn<R><<<(td_.nwin + 255) / 256, 256, 0, st_>>>(tctl_, td_.f_n, F_[LESGO_FXA], F_[LESGO_FYA],
                                                                      fza_uv_);
      else
        k_turb_scatter<R><<<(td_.nwin + 255) / 256, 256, 0, st_>>>(td_, F_[LESGO_FXA], F_[LESGO_FYA], fza_uv_);
      post("turbines.scatter", (double)td_.nwin * (3 * sizeof(R) + 20.0));
      const long long n = (long long)th_.cols.size() * d_.nz;
      pre();
      k_turb_fzw<R><<<grid1(n), 256, 0, st_>>>(fza_uv_, F_[LESGO_FZA], cols_, (int)th_.cols.size(), kp_);
      post("turbines.fzw", 2.0 * n * sizeof(R));
    }
  }

  Derived d_;
  int cap_ = 1;
  KP kp_{};
  cudaStream_t st_ = nullptr;
  std::vector<void*> allocs_;
  std::vector<Slot> slots_;
  int next_id_ = 0;
  long long nfield_ = 0, vol1_s_ = 0, vol1_b_ = 0;
  R* F_[LESGO_NFIELDS] = {};
  R* Ftmp_[4] = {};
  R* wall_[4] = {};
  R* big_[6] = {};
  R* fza_uv_ = nullptr;
  T2 *specA_ = nullptr, *specB_ = nullptr, *specC_ = nullptr;
  double2 *hspec_ = nullptr, *hplane_ = nullptr, *phat_ = nullptr;
  double *ibet_ = nullptr, *tgam_ = nullptr;
  double *tacc_ = nullptr, *tw_d_ = nullptr, *prof_d_ = nullptr;
  double* sc_d_ = nullptr;                   // step constants [cap][SC_N]
  T2 *cvA_ = nullptr, *cvB_ = nullptr;       // convective-term spectra
  cudaStream_t st2_ = nullptr;               // second branch of the fused step
  cudaEvent_t ev_[8] = {};
  static constexpr int kRing = 64;
  int* ring_h_ = nullptr;                    // pinned [kRing][cap]
  cudaEvent_t ring_ev_[kRing] = {};
  long long ring_next_ = 0;
  unsigned long long* cflmax_d_ = nullptr;   // per-instance |u|, |v|, |w| maxima
  int* tact_d_ = nullptr;                    // time-averaging action per instance
  double* dlog_ = nullptr;                   // diagnostics log [cap][dlog_cap_][6]
  // tile shapes: complex values per block of the x passes, shared-memory
  // bytes per block of the y passes
  int xtarget_ = 2048;
  size_t ybudget_ = sizeof(T2) == 16 ? 110 * 1024 : 48 * 1024;
  int ythreads_ = 256;   // y-pass block size (a multiple of the tile width)
  bool yshort_ = true;   // y-pass outputs without transforms where the operator allows (k_ypass)
  int thomas_mode_ = 0;   // 0 by column count, 1 sequential, 2 segmented
  int dlog_cap_ = 0, dlog_every_ = 0;
  long long tacc_stride_ = 0;
  bool tavg_on_ = false;
  int ta_nstart_ = 1, ta_nend_ = 50000, ta_nskip_ = 100;
  int* err_ = nullptr;
  double* zo_d_ = nullptr;
  int* flags_d_ = nullptr;
  double *diag_part_ = nullptr, *diag_out_ = nullptr;
  double* staging_ = nullptr;
  long long staging_n_ = 0;
  FftPlan<A> px_{}, py_{}, pxb_{}, pyb_{};
  A *kxw_ = nullptr, *kyw_ = nullptr, *G1_ = nullptr, *G2_ = nullptr;
  int kmax_g_[2] = {1 << 30, 1 << 30};   // largest kx column with a nonzero G1 / G2 weight
  double *kxw64_ = nullptr, *kyw64_ = nullptr;
  TurbineHost th_;
  TurbDev td_{};
  TurbDyn tctl_{};
  std::vector<void*> turb_allocs_;
  IndicatorCache ind_cache_;
  std::map<int, int> turb_base_;
  long long* cols_ = nullptr;
  double* tri_gam_ = nullptr;
  long long tri_gam_n_ = 0;
  bool use_graphs_ = true, graphs_allowed_ = true;
  int launches_ = 0;
  bool prof_on_ = false;
  bool branches_allowed_ = true;   // LESGO_BRANCHES=0: the fused step on one stream
  bool conv_rows_ = false;         // the one-pass 3/2-grid x-rows of the convective term
  float* xdft_w_ = nullptr;        // DFT matrix images of the tensor-core x transform (when enabled)
  cudaEvent_t prof_start_ = nullptr;
  std::vector<ProfRec> prof_;
  std::map<int, cudaGraphExec_t> graphs_;
  std::map<int, int> launch_count_;
};

// Factories of the precision forms, one per translation unit.
SolverBase* make_solver_fp32(const Derived& d, int capacity);
SolverBase* make_solver_fp64(const Derived& d, int capacity);
SolverBase* make_solver_dw(const Derived& d, int capacity);

}  // namespace lesgo

// The C ABI declared in include/lesgo_gpu.h.
#include "solver_impl.cuh"

namespace lesgo {

// The solver of a precision form.
static SolverBase* make_solver(const Derived& d, int capacity) {
  switch (d.p.precision) {
    case LESGO_FP64: return make_solver_fp64(d, capacity);
    case LESGO_FP64_DW: return make_solver_dw(d, capacity);
    default: return make_solver_fp32(d, capacity);
  }
}

}  // namespace lesgo


// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
struct lesgo_handle {
  std::unique_ptr<lesgo::SolverBase> s;
  int inst0 = -1;   // the instance of a single-instance handle (lesgo_gpu_create)
  std::string err;
  struct Bind { double* ptr = nullptr; int lbz = 0, nzhi = -1; };
  Bind bind[LESGO_NFIELDS];
};

static thread_local std::string g_create_err;

template <typename F>
static int guarded(lesgo_handle_t* h, F&& fn) {
  if (!h || !h->s) return LESGO_ERR_ARG;
  try {
    fn();
    return LESGO_OK;
  } catch (const lesgo::Error& e) {
    h->err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    h->err = e.what();
    return LESGO_ERR_CUDA;
  }
}

extern "C" {

int lesgo_gpu_params_default(lesgo_params_t* p) {
  if (!p) return LESGO_ERR_ARG;
  std::memset(p, 0, sizeof(*p));
  p->nx = 64; p->ny = 64; p->nz_tot = 64;
  p->L_x = 2.0 * 3.1415926535897932384626433; p->L_y = 3.1415926535897932384626433; p->L_z = 1.0; p->z_i = 1000.0;
  p->u_star = 0.45; p->vonk = 0.4; p->zo = 1.0e-4; p->dt = 2.0e-4;
  p->sgs_model = 5; p->cs_count = 5; p->dyn_init = 100; p->ifilter = 1;
  p->lbc_mom = 2; p->ubc_mom = 0;
  p->molec = 0; p->nu_molec = 1.14e-5;
  p->use_mean_p_force = 1; p->eval_mean_p_force = 1;
  p->mean_p_force_x = 1.0; p->mean_p_force_y = 0.0;
  p->precision = LESGO_FP64;
  p->alpha1 = 1.5; p->alpha2 = 1.5; p->filter_cutoff = 1e-2; p->T_avg_dim = -1.0; p->adm_correction = 1;
  p->use_cfl_dt = 0; p->cfl = (double)0.05f;
  return LESGO_OK;
}

int lesgo_gpu_create(const lesgo_params_t* p, lesgo_handle_t** h) {
  if (!p || !h) return LESGO_ERR_ARG;
  *h = nullptr;
  try {
    lesgo::Derived d(*p);
    auto* hh = new lesgo_handle;
    try {
      hh->s.reset(lesgo::make_solver(d, 1));
      lesgo::InstanceSpec spec{p->zo, 0, d.turbines};
      hh->inst0 = hh->s->add_instance(spec);
    } catch (...) {
      delete hh;
      throw;
    }
    *h = hh;
    return LESGO_OK;
  } catch (const lesgo::Error& e) {
    g_create_err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    g_create_err = e.what();
    return LESGO_ERR_CUDA;
  }
}

int lesgo_gpu_destroy(lesgo_handle_t* h) {
  if (!h) return LESGO_ERR_ARG;
  delete h;
  return LESGO_OK;
}

const char* lesgo_gpu_last_error(const lesgo_handle_t* h) {
  if (!h) return g_create_err.c_str();
  return h->err.c_str();
}

int lesgo_gpu_dims(const lesgo_handle_t* h, int* nz, int* ld, int* lh, int* nx2, int* ny2) {
  if (!h || !h->s) return LESGO_ERR_ARG;
  const auto& d = h->s->der();
  if (nz) *nz = d.nz;
  if (ld) *ld = d.ld;
  if (lh) *lh = d.lh;
  if (nx2) *nx2 = d.nx2;
  if (ny2) *ny2 = d.ny2;
  return LESGO_OK;
}

int lesgo_gpu_set_field(lesgo_handle_t* h, int f, const double* host, int lbz, int nzhi) {
  if (!host) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->set_field(h->inst0, f, host, lbz, nzhi); });
}
int lesgo_gpu_get_field(lesgo_handle_t* h, int f, double* host, int lbz, int nzhi) {
  if (!host) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->get_field(h->inst0, f, host, lbz, nzhi); });
}
int lesgo_gpu_set_field_async(lesgo_handle_t* h, int f, const double* host, int lbz, int nzhi) {
  if (!host) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->set_field(h->inst0, f, host, lbz, nzhi, false); });
}
int lesgo_gpu_get_field_async(lesgo_handle_t* h, int f, double* host, int lbz, int nzhi) {
  if (!host) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->get_field(h->inst0, f, host, lbz, nzhi, false); });
}
int lesgo_gpu_bind_field(lesgo_handle_t* h, int f, double* host, int lbz, int nzhi) {
  if (!h || !h->s || !host || f < 0 || f >= LESGO_NFIELDS) return LESGO_ERR_ARG;
  if (lbz < 0 || nzhi > h->s->der().nz || nzhi < lbz) return LESGO_ERR_ARG;
  h->bind[f].ptr = host; h->bind[f].lbz = lbz; h->bind[f].nzhi = nzhi;
  return LESGO_OK;
}
int lesgo_gpu_upload(lesgo_handle_t* h, int f) {
  if (!h || f < 0 || f >= LESGO_NFIELDS || !h->bind[f].ptr) return LESGO_ERR_ARG;
  return lesgo_gpu_set_field(h, f, h->bind[f].ptr, h->bind[f].lbz, h->bind[f].nzhi);
}
int lesgo_gpu_download(lesgo_handle_t* h, int f) {
  if (!h || f < 0 || f >= LESGO_NFIELDS || !h->bind[f].ptr) return LESGO_ERR_ARG;
  return lesgo_gpu_get_field(h, f, h->bind[f].ptr, h->bind[f].lbz, h->bind[f].nzhi);
}
int lesgo_gpu_init_ic(lesgo_handle_t* h, uint64_t seed) { return guarded(h, [&] { h->s->init_ic(h->inst0, seed); }); }

static bool fid_ok(int f) { return f >= 0 && f < LESGO_NFIELDS; }

int lesgo_gpu_filt_da(lesgo_handle_t* h, int f, int dfdx, int dfdy) {
  if (!fid_ok(f) || !fid_ok(dfdx) || !fid_ok(dfdy)) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->filt_da(f, dfdx, dfdy); });
}
int lesgo_gpu_ddx(lesgo_handle_t* h, int f, int dfdx) {
  if (!fid_ok(f) || !fid_ok(dfdx)) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->ddxy(f, dfdx, -1); });
}
int lesgo_gpu_ddy(lesgo_handle_t* h, int f, int dfdy) {
  if (!fid_ok(f) || !fid_ok(dfdy)) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->ddxy(f, -1, dfdy); });
}
int lesgo_gpu_ddxy(lesgo_handle_t* h, int f, int dfdx, int dfdy) {
  if (!fid_ok(f) || !fid_ok(dfdx) || !fid_ok(dfdy)) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->ddxy(f, dfdx, dfdy); });
}
int lesgo_gpu_ddz_uv(lesgo_handle_t* h, int f, int dfdz) {
  if (!fid_ok(f) || !fid_ok(dfdz)) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->ddz(f, dfdz, true); });
}
int lesgo_gpu_ddz_w(lesgo_handle_t* h, int f, int dfdz) {
  if (!fid_ok(f) || !fid_ok(dfdz)) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->ddz(f, dfdz, false); });
}
int lesgo_gpu_test_filter(lesgo_handle_t* h, int f, int level) {
  if (!fid_ok(f)) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->test_filter(f, level); });
}
int lesgo_gpu_wallstress(lesgo_handle_t* h) { return guarded(h, [&] { h->s->wallstress(); }); }
int lesgo_gpu_sgs_stag(lesgo_handle_t* h) { return guarded(h, [&] { h->s->sgs_stag(); }); }
int lesgo_gpu_divstress_uv(lesgo_handle_t* h) { return guarded(h, [&] { h->s->divstress(1); }); }
int lesgo_gpu_divstress_w(lesgo_handle_t* h) { return guarded(h, [&] { h->s->divstress(2); }); }
int lesgo_gpu_convec(lesgo_handle_t* h) { return guarded(h, [&] { h->s->convec(); }); }
int lesgo_gpu_turbines_forcing(lesgo_handle_t* h) { return guarded(h, [&] { h->s->turbines_forcing(); }); }
int lesgo_gpu_begin_step(lesgo_handle_t* h) { return guarded(h, [&] { h->s->begin_step(); }); }
int lesgo_gpu_rhs_assemble(lesgo_handle_t* h) { return guarded(h, [&] { h->s->rhs_assemble(); }); }
int lesgo_gpu_ab2(lesgo_handle_t* h) { return guarded(h, [&] { h->s->ab2(); }); }
int lesgo_gpu_press_stag_array(lesgo_handle_t* h) { return guarded(h, [&] { h->s->press_stag_array(); }); }
int lesgo_gpu_rhs_sub_dp(lesgo_handle_t* h) { return guarded(h, [&] { h->s->rhs_sub_dp(); }); }
int lesgo_gpu_project(lesgo_handle_t* h) { return guarded(h, [&] { h->s->project(); }); }
int lesgo_gpu_step(lesgo_handle_t* h, int nsteps) {
  if (nsteps < 0) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->step(nsteps); });
}
int lesgo_gpu_sync(lesgo_handle_t* h) {
  int rc = LESGO_OK;
  int g = guarded(h, [&] { rc = h->s->sync(); });
  if (g != LESGO_OK) return g;
  if (rc != LESGO_OK) h->err = "tridag_array: zero pivot";
  return rc;
}
int lesgo_gpu_diag(lesgo_handle_t* h, double* rmsdiv, double* ke, double* cfl, double* tau_bot) {
  double out[4] = {0, 0, 0, 0};
  int rc = guarded(h, [&] { h->s->diag(h->inst0, out); });
  if (rc == LESGO_OK) {
    if (rmsdiv) *rmsdiv = out[0];
    if (ke) *ke = out[1];
    if (cfl) *cfl = out[2];
    if (tau_bot) *tau_bot = out[3];
  }
  return rc;
}
int lesgo_gpu_counters(const lesgo_handle_t* h, int* jt, int* jt_total) {
  if (!h || !h->s) return LESGO_ERR_ARG;
  try {
    h->s->counters(h->inst0, jt, jt_total);
  } catch (...) {
    return LESGO_ERR_ARG;
  }
  return LESGO_OK;
}
int lesgo_gpu_turbine_state(lesgo_handle_t* h, double* u_d_T, double* f_n, double* power, int n) {
  if (n < 0) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->turbine_state(h->inst0, u_d_T, f_n, power, n); });
}
int lesgo_gpu_launches_per_step(const lesgo_handle_t* h, int with_sgs_update) {
  if (!h || !h->s) return -1;
  return h->s->launches_per_step(with_sgs_update);
}

}  // extern "C"

extern "C" {
int lesgo_gpu_profile(lesgo_handle_t* h, int enable) { return guarded(h, [&] { h->s->profile(enable); }); }
int lesgo_gpu_profile_report(lesgo_handle_t* h, char* buf, int buflen) {
  if (!buf || buflen <= 0) return LESGO_ERR_ARG;
  std::string r;
  int rc = guarded(h, [&] { r = h->s->profile_report(); });
  if (rc != LESGO_OK) return rc;
  if ((int)r.size() + 1 > buflen) return LESGO_ERR_ARG;
  std::memcpy(buf, r.c_str(), r.size() + 1);
  return LESGO_OK;
}
int lesgo_gpu_get_stream(const lesgo_handle_t* h, void** stream) {
  if (!h || !h->s || !stream) return LESGO_ERR_ARG;
  *stream = h->s->stream();
  return LESGO_OK;
}
}  // extern "C"

extern "C" int lesgo_gpu_tridag_array(lesgo_handle_t* h, const double* a, const double* b, const double* c,
                                      const double* r, double* u, int lh, int ny, int n) {
  if (!a || !b || !c || !r || !u || lh < 2 || ny < 1 || n < 1) return LESGO_ERR_ARG;
  int rc = LESGO_OK;
  int g = guarded(h, [&] { rc = h->s->tridag(a, b, c, r, u, lh, ny, n); });
  if (g != LESGO_OK) return g;
  if (rc != LESGO_OK) h->err = "tridag_array: zero pivot";
  return rc;
}

// ---------------------------------------------------------------------------
// Allocation-free tridiagonal solve.
//
// lesgo_gpu_tridag_array_noalloc runs the same Thomas kernel as
// lesgo_gpu_tridag_array but takes its scratch from a fixed array compiled
// into this library instead of asking the CUDA allocator.  It serves
// callers that must not allocate device memory themselves: code that owns
// every device buffer through its own pool or framework, loops that must not
// stall on cudaMalloc/cudaFree (which can synchronise the device), and
// callers that hold no solver handle at all.
//
// The scratch array is a file-scope __device__ array of kTridagScratchDoubles
// doubles (16 MiB); every GPU that loads the library holds it until the
// process exits.  Host code may not use the array's name as a device
// address, so the first call on each device looks the address up with
// cudaGetSymbolAddress while that device is current and caches it.  No call
// can be captured in a CUDA graph (each waits for its own result): a call on
// a capturing stream returns LESGO_ERR_ARG without queueing anything.  All
// calls on a device share the
// array and it keeps the previous call's contents (the solve writes every
// scratch entry before reading it; the error flag is cleared each call), so
// calls whose GPU work overlaps in time race on it: issue them in order, on
// one stream or with events between them.
// ---------------------------------------------------------------------------
namespace {
constexpr long long kTridagScratchDoubles = 1LL << 21;
__device__ __align__(256) double g_tridag_scratch[kTridagScratchDoubles];
__device__ __align__(256) int g_tridag_err;

struct NoAllocSlot { double* scratch = nullptr; int* err = nullptr; };
std::mutex g_noalloc_mu;
std::map<int, NoAllocSlot> g_noalloc_slots;

int noalloc_fail(int code, const std::string& msg) {
  g_create_err = msg;
  return code;
}
}  // namespace

extern "C" int lesgo_gpu_tridag_array_noalloc(const double* a, const double* b, const double* c, const double* r,
                                              double* u, int lh, int ny, int n, void* stream) {
  if (!a || !b || !c || !r || !u || lh < 2 || ny < 1 || n < 1)
    return noalloc_fail(LESGO_ERR_ARG, "tridag_array_noalloc: null pointer or bad size");
  const long long need = (long long)lh * ny * n;
  if (need > kTridagScratchDoubles)
    return noalloc_fail(LESGO_ERR_ARG, "tridag_array_noalloc: lh*ny*n = " + std::to_string(need) +
                                           " exceeds the fixed scratch of " + std::to_string(kTridagScratchDoubles) +
                                           " doubles");
  // the call reads its pivot flag back and waits for the stream, which a
  // capturing stream cannot do: refuse before queueing anything, so that
  // the caller's capture stays intact
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing((cudaStream_t)stream, &cap);
  if (e != cudaSuccess)
    return noalloc_fail(LESGO_ERR_CUDA, std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(e));
  if (cap != cudaStreamCaptureStatusNone)
    return noalloc_fail(LESGO_ERR_ARG, "tridag_array_noalloc: the stream is capturing; the call waits for its "
                                       "result, so it cannot be captured");
  int dev = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(LESGO_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  NoAllocSlot slot;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    auto it = g_noalloc_slots.find(dev);
    if (it == g_noalloc_slots.end()) {
      NoAllocSlot s;
      e = cudaGetSymbolAddress((void**)&s.scratch, g_tridag_scratch);
      if (e != cudaSuccess)
        return noalloc_fail(LESGO_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
      e = cudaGetSymbolAddress((void**)&s.err, g_tridag_err);
      if (e != cudaSuccess)
        return noalloc_fail(LESGO_ERR_CUDA, std::string("cudaGetSymbolAddress(flag): ") + cudaGetErrorString(e));
      it = g_noalloc_slots.emplace(dev, s).first;
    }
    slot = it->second;
  }
  cudaStream_t st = (cudaStream_t)stream;
  e = cudaMemsetAsync(slot.err, 0, sizeof(int), st);
  if (e != cudaSuccess) return noalloc_fail(LESGO_ERR_CUDA, std::string("clear flag: ") + cudaGetErrorString(e));
  const int ncol = (lh - 1) * ny;
  lesgo::k_tridag<<<(ncol + 127) / 128, 128, 0, st>>>(a, b, c, (const double2*)r, (double2*)u, slot.scratch, lh, ny, n,
                                                        slot.err);
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(LESGO_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  int flag = 0;
  e = cudaMemcpyAsync(&flag, slot.err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return noalloc_fail(LESGO_ERR_CUDA, std::string("tridag_array_noalloc: ") + cudaGetErrorString(e));
  if (flag) return noalloc_fail(LESGO_ERR_NUMERIC, "tridag_array_noalloc: zero pivot");
  return LESGO_OK;
}

// ---------------------------------------------------------------------------
// Batches of independent instances of one grid size
// ---------------------------------------------------------------------------
extern "C" {

int lesgo_gpu_batch_create(const lesgo_params_t* p, int capacity, lesgo_handle_t** h) {
  if (!p || !h || capacity < 1) return LESGO_ERR_ARG;
  *h = nullptr;
  try {
    lesgo::Derived d(*p);
    auto* hh = new lesgo_handle;
    try {
      hh->s.reset(lesgo::make_solver(d, capacity));
    } catch (...) {
      delete hh;
      throw;
    }
    *h = hh;
    return LESGO_OK;
  } catch (const lesgo::Error& e) {
    g_create_err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    g_create_err = e.what();
    return LESGO_ERR_CUDA;
  }
}

int lesgo_gpu_batch_add(lesgo_handle_t* h, double zo, uint64_t seed, int n_turbines, const lesgo_turbine_t* turbines,
                        int* id) {
  if (!id || n_turbines < 0 || (n_turbines > 0 && !turbines)) return LESGO_ERR_ARG;
  return guarded(h, [&] {
    lesgo::InstanceSpec spec{zo, seed, std::vector<lesgo_turbine_t>(turbines, turbines + n_turbines)};
    *id = h->s->add_instance(spec);
  });
}

int lesgo_gpu_batch_remove(lesgo_handle_t* h, int id) { return guarded(h, [&] { h->s->remove_instance(id); }); }

int lesgo_gpu_batch_size(const lesgo_handle_t* h, int* active, int* capacity) {
  if (!h || !h->s) return LESGO_ERR_ARG;
  if (active) *active = h->s->active();
  if (capacity) *capacity = h->s->capacity();
  return LESGO_OK;
}

int lesgo_gpu_set_field_inst(lesgo_handle_t* h, int id, int f, const double* host, int lbz, int nzhi) {
  if (!host) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->set_field(id, f, host, lbz, nzhi); });
}
int lesgo_gpu_get_field_inst(lesgo_handle_t* h, int id, int f, double* host, int lbz, int nzhi) {
  if (!host) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->get_field(id, f, host, lbz, nzhi); });
}
int lesgo_gpu_set_field_inst_async(lesgo_handle_t* h, int id, int f, const double* host, int lbz, int nzhi) {
  if (!host) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->set_field(id, f, host, lbz, nzhi, false); });
}
int lesgo_gpu_get_field_inst_async(lesgo_handle_t* h, int id, int f, double* host, int lbz, int nzhi) {
  if (!host) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->get_field(id, f, host, lbz, nzhi, false); });
}
int lesgo_gpu_turbine_schedule(lesgo_handle_t* h, int which, int nt, const double* rows) {
  return guarded(h, [&] { h->s->turbine_schedule(h->inst0, which, nt, rows); });
}
int lesgo_gpu_turbine_schedule_inst(lesgo_handle_t* h, int id, int which, int nt, const double* rows) {
  return guarded(h, [&] { h->s->turbine_schedule(id, which, nt, rows); });
}
int lesgo_gpu_turbine_controls(lesgo_handle_t* h, int id, double* theta1, double* theta2, double* ct_prime, int n) {
  return guarded(h, [&] { h->s->turbine_controls(id < 0 ? h->inst0 : id, theta1, theta2, ct_prime, n); });
}
int lesgo_gpu_diag_inst(lesgo_handle_t* h, int id, double* rmsdiv, double* ke, double* cfl, double* tau_bot) {
  double out[4] = {0, 0, 0, 0};
  int rc = guarded(h, [&] { h->s->diag(id, out); });
  if (rc == LESGO_OK) {
    if (rmsdiv) *rmsdiv = out[0];
    if (ke) *ke = out[1];
    if (cfl) *cfl = out[2];
    if (tau_bot) *tau_bot = out[3];
  }
  return rc;
}
int lesgo_gpu_counters_inst(lesgo_handle_t* h, int id, int* jt, int* jt_total) {
  return guarded(h, [&] { h->s->counters(id, jt, jt_total); });
}
int lesgo_gpu_turbine_state_inst(lesgo_handle_t* h, int id, double* u_d_T, double* f_n, double* power, int n) {
  if (n < 0) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->turbine_state(id, u_d_T, f_n, power, n); });
}
int lesgo_gpu_footprint(const lesgo_params_t* p, int capacity, long long* bytes) {
  if (!p || !bytes || capacity < 1) return LESGO_ERR_ARG;
  try {
    lesgo::Derived d(*p);
    *bytes = lesgo::footprint_bytes(d, capacity);
    return LESGO_OK;
  } catch (const lesgo::Error& e) {
    g_create_err = e.what();
    return e.code;
  }
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Time-averaging statistics
// ---------------------------------------------------------------------------
extern "C" {
int lesgo_gpu_tavg_config(lesgo_handle_t* h, int nstart, int nend, int nskip) {
  return guarded(h, [&] { h->s->tavg_config(nstart, nend, nskip); });
}
int lesgo_gpu_tavg_sample(lesgo_handle_t* h) { return guarded(h, [&] { h->s->tavg_sample(); }); }
int lesgo_gpu_tavg_get(lesgo_handle_t* h, int which, double* host, int lbz, int nzhi) {
  if (!host) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->tavg_get(h->inst0, which, host, lbz, nzhi); });
}
int lesgo_gpu_tavg_get_inst(lesgo_handle_t* h, int id, int which, double* host, int lbz, int nzhi) {
  if (!host) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->tavg_get(id, which, host, lbz, nzhi); });
}
int lesgo_gpu_tavg_profile(lesgo_handle_t* h, int which, double* prof, int n) {
  if (!prof) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->tavg_profile(h->inst0, which, prof, n); });
}
int lesgo_gpu_tavg_profile_inst(lesgo_handle_t* h, int id, int which, double* prof, int n) {
  if (!prof) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->tavg_profile(id, which, prof, n); });
}
int lesgo_gpu_tavg_total_time(lesgo_handle_t* h, int id, double* t) {
  if (!t) return LESGO_ERR_ARG;
  return guarded(h, [&] { *t = h->s->tavg_total_time(id < 0 ? h->inst0 : id); });
}
}  // extern "C"

// ---------------------------------------------------------------------------
// Checkpoint / restart files
// ---------------------------------------------------------------------------
extern "C" {
int lesgo_gpu_checkpoint_write(lesgo_handle_t* h, const char* path, int mpi_names) {
  if (!path) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->checkpoint_write(h->inst0, path, mpi_names); });
}
int lesgo_gpu_checkpoint_write_inst(lesgo_handle_t* h, int id, const char* path, int mpi_names) {
  if (!path) return LESGO_ERR_ARG;
  return guarded(h, [&] { h->s->checkpoint_write(id, path, mpi_names); });
}
int lesgo_gpu_checkpoint_read(lesgo_handle_t* h, const char* path, int* same_grid) {
  if (!path) return LESGO_ERR_ARG;
  return guarded(h, [&] {
    const int e = h->s->checkpoint_read(h->inst0, path);
    if (same_grid) *same_grid = e;
  });
}
int lesgo_gpu_checkpoint_read_inst(lesgo_handle_t* h, int id, const char* path, int* same_grid) {
  if (!path) return LESGO_ERR_ARG;
  return guarded(h, [&] {
    const int e = h->s->checkpoint_read(id, path);
    if (same_grid) *same_grid = e;
  });
}
int lesgo_gpu_sim_time(lesgo_handle_t* h, int id, double* total_time) {
  if (!total_time) return LESGO_ERR_ARG;
  return guarded(h, [&] { *total_time = h->s->sim_time(id < 0 ? h->inst0 : id); });
}
int lesgo_gpu_time_step(lesgo_handle_t* h, int id, double* dt) {
  if (!dt) return LESGO_ERR_ARG;
  return guarded(h, [&] { *dt = h->s->time_step(id < 0 ? h->inst0 : id); });
}
}  // extern "C"

// ---------------------------------------------------------------------------
// lesgo.conf
// ---------------------------------------------------------------------------
extern "C" int lesgo_gpu_read_conf(const char* path, int with_turbines, lesgo_params_t* p, lesgo_run_t* run,
                                   lesgo_turbine_t* turbines, int max_turbines, char* log, int loglen) {
  if (!path || !p || !run || (with_turbines && max_turbines > 0 && !turbines)) return LESGO_ERR_ARG;
  try {
    std::string lg;
    lesgo::conf::read(path, with_turbines, p, run, turbines, with_turbines ? max_turbines : 0, &lg);
    if (log && loglen > 0) {
      std::strncpy(log, lg.c_str(), (size_t)loglen - 1);
      log[loglen - 1] = '\0';
    }
    return LESGO_OK;
  } catch (const lesgo::conf::ConfError& e) {
    g_create_err = e.msg;
    return e.code;
  } catch (const std::exception& e) {
    g_create_err = e.what();
    return LESGO_ERR_ARG;
  }
}

extern "C" int lesgo_gpu_read_turbine_schedule(const char* path, int which, int n_turbines, double* rows,
                                               int max_rows, int* nt) {
  if (!path || !nt || (max_rows > 0 && !rows) || max_rows < 0) return LESGO_ERR_ARG;
  try {
    const std::vector<double> v = lesgo::conf::read_schedule(path, which, n_turbines);
    const int n = (int)(v.size() / (1 + n_turbines));
    if (n > max_rows) {
      g_create_err = "schedule holds " + std::to_string(n) + " rows, buffer " + std::to_string(max_rows);
      return LESGO_ERR_ARG;
    }
    std::copy(v.begin(), v.end(), rows);
    *nt = n;
    return LESGO_OK;
  } catch (const lesgo::conf::ConfError& e) {
    g_create_err = e.msg;
    return e.code;
  }
}

// ---------------------------------------------------------------------------
// Diagnostics log
// ---------------------------------------------------------------------------
extern "C" {
int lesgo_gpu_diag_log_config(lesgo_handle_t* h, int every, int capacity) {
  return guarded(h, [&] { h->s->diag_log_config(every, capacity); });
}
int lesgo_gpu_diag_log_sample(lesgo_handle_t* h) { return guarded(h, [&] { h->s->diag_log_sample(); }); }
int lesgo_gpu_diag_log_read(lesgo_handle_t* h, int id, double* rows, int maxrows, int* nrows) {
  if (!rows || !nrows || maxrows < 0) return LESGO_ERR_ARG;
  return guarded(h, [&] { *nrows = h->s->diag_log_read(id < 0 ? h->inst0 : id, rows, maxrows); });
}
}  // extern "C"

extern "C" int lesgo_gpu_autotune(lesgo_handle_t* h, int* xtarget, int* ybudget) {
  return guarded(h, [&] { h->s->autotune(xtarget, ybudget); });
}

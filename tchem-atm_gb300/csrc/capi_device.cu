// C ABI: device entry points (time advance, unit kernels, workspace planning).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "advance.hpp"
#include "capi_internal.hpp"
#include "kernels.hpp"
#include "kernels_mixed.hpp"
#include "mech_host.hpp"

namespace tchem_gb {

DeviceInfo device_info(int dev) {
  static std::mutex mu;
  static std::vector<DeviceInfo> cache;
  std::lock_guard<std::mutex> lk(mu);
  if (static_cast<int>(cache.size()) <= dev) cache.resize(dev + 1);
  if (cache[dev].sm_count == 0) {
    cudaDeviceGetAttribute(&cache[dev].sm_count, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&cache[dev].max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  }
  return cache[dev];
}

DeviceTables* tables_for(const tchem_gb_mech* mech, int dev) {
  auto* m = const_cast<tchem_gb_mech*>(mech);
  std::lock_guard<std::mutex> lk(m->mu);
  if (!m->host_tables) m->host_tables.reset(new HostTables(build_host_tables(m->km)));
  if (static_cast<int>(m->device_tables.size()) <= dev) m->device_tables.resize(dev + 1, nullptr);
  if (!m->device_tables[dev]) m->device_tables[dev] = upload_tables(*m->host_tables, dev);
  return m->device_tables[dev];
}

// Library-owned workspace per device (used when the caller passes none).
namespace {
struct OwnedWorkspace {
  void* ptr = nullptr;
  size_t bytes = 0;
};
std::mutex g_ws_mu;
std::vector<OwnedWorkspace> g_ws;
}  // namespace

void* owned_workspace(int dev, size_t bytes) {
  std::lock_guard<std::mutex> lk(g_ws_mu);
  if (static_cast<int>(g_ws.size()) <= dev) g_ws.resize(dev + 1);
  OwnedWorkspace& w = g_ws[dev];
  if (w.bytes < bytes) {
    if (w.ptr) {
      cudaDeviceSynchronize();
      cudaFree(w.ptr);
      w.ptr = nullptr;
      w.bytes = 0;
    }
    const size_t want = std::max(bytes, size_t(1) << 20);
    if (cudaMalloc(&w.ptr, want) != cudaSuccess) {
      cudaGetLastError();
      throw std::bad_alloc();
    }
    // the header's device error word persists until tchem_gb_device_error reads it: start clear
    if (cudaMemset(w.ptr, 0, kHeaderBytes) != cudaSuccess) {
      cudaGetLastError();
      cudaFree(w.ptr);
      w.ptr = nullptr;
      throw std::bad_alloc();
    }
    w.bytes = want;
  }
  return w.ptr;
}

void* owned_workspace_peek(int dev) {
  std::lock_guard<std::mutex> lk(g_ws_mu);
  return static_cast<int>(g_ws.size()) > dev ? g_ws[dev].ptr : nullptr;
}

namespace {
// Library-owned side streams and events per device: the kernels of a batch's mechanism-structure
// groups run concurrently, forked from and joined back into the caller's stream.
constexpr int kSideStreams = 15;  // groups beyond the first (kMaxGroups - 1)
struct SideStreams {
  cudaStream_t s[kSideStreams] = {};
  cudaEvent_t fork = nullptr, join[kSideStreams] = {};
  bool ready = false;
  std::mutex mu;  // held from the fork to the join of one call
};
std::mutex g_side_mu;
std::vector<std::unique_ptr<SideStreams>> g_side;

// The device's side streams (created on first use); nullptr when creation failed.
SideStreams* side_streams(int dev) {
  std::lock_guard<std::mutex> lk(g_side_mu);
  while (static_cast<int>(g_side.size()) <= dev) g_side.emplace_back(new SideStreams());
  SideStreams& ss = *g_side[dev];
  if (!ss.ready) {
    bool ok = cudaEventCreateWithFlags(&ss.fork, cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; i < kSideStreams && ok; ++i)
      ok = cudaStreamCreateWithFlags(&ss.s[i], cudaStreamNonBlocking) == cudaSuccess &&
           cudaEventCreateWithFlags(&ss.join[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      return nullptr;
    }
    ss.ready = true;
  }
  return &ss;
}
}  // namespace

int fail(int code, const std::string& msg) {
  set_last_error(msg);
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(TCHEM_GB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

namespace {
std::atomic<long long> g_kernel_launches{0};
}  // namespace

void note_launch(int n) { g_kernel_launches.fetch_add(n, std::memory_order_relaxed); }

namespace {

constexpr int kMaxGroups = 16;
constexpr int kMaxWarpsPerBlock = 8;

size_t up256(size_t b) { return (b + 255) & ~size_t(255); }

struct GroupPlan {
  std::vector<int> mechs;  // global mechanism indices in slot order
  MechDev dev{};
  const void* kernel = nullptr;
  int form = 0;
  int warps_per_block = 0;
  int grid = 0;
  size_t smem = 0;
  int lda = 0;
  bool matrix_in_smem = true;
  uint32_t warp_smem = 0;
  size_t gmat_offset = 0;
  size_t gmat_elems_per_warp = 0;
  int threads_per_sample = 32;
  bool tc = false;  // the tensor-core form (kernels_tc_advance.cu)
  MixedLayout ml{};
};

struct Plan {
  std::vector<GroupPlan> groups;
  bool need_items = false;
  size_t items_offset = 0;
  size_t bytes = 0;
  int m_max = 0;
};

// Groups structurally identical mechanisms and sizes each group's launch.
// e3sm: the E3SM time advance (per-sample rate constants and source terms): every rate form of
// the E3SM tables is allowed, and each warp group gets a source-term section.
Plan make_plan(const tchem_gb_mech* const* mechs, int n_mechs, int nbatch, bool have_mos, const tchem_gb_advance_opts& o,
               int dev, bool e3sm = false) {
  if (n_mechs <= 0 || n_mechs > kMaxMechs) throw std::invalid_argument("n_mechs must be in [1, 64]");
  Plan plan;
  std::vector<const HostTables*> hts(n_mechs);
  std::vector<DeviceTables*> dts(n_mechs);
  for (int i = 0; i < n_mechs; ++i) {
    if (!mechs[i]) throw std::invalid_argument("null mechanism handle");
    dts[i] = tables_for(mechs[i], dev);
    hts[i] = mechs[i]->host_tables.get();
    if (e3sm) {
      if (!hts[i]->e3sm_valid) throw std::domain_error(hts[i]->e3sm_invalid_reason);
      if (!hts[i]->e3sm_state_free) throw std::domain_error(hts[i]->e3sm_reason);
    } else if (!hts[i]->supported) {
      throw std::domain_error(hts[i]->unsupported_reason);
    }
  }
  for (int i = 0; i < n_mechs; ++i) {
    bool placed = false;
    for (auto& g : plan.groups) {
      if (static_cast<int>(g.mechs.size()) < kMaxGroupSlots && hts[g.mechs[0]]->signature == hts[i]->signature) {
        g.mechs.push_back(i);
        placed = true;
        break;
      }
    }
    if (!placed) {
      if (static_cast<int>(plan.groups.size()) >= kMaxGroups) throw std::invalid_argument("too many mechanism groups");
      GroupPlan g;
      g.mechs.push_back(i);
      g.dev = dts[i]->dev;
      plan.groups.push_back(g);
    }
  }
  plan.need_items = have_mos && plan.groups.size() > 1;
  size_t off = kHeaderBytes;
  if (plan.need_items) {
    plan.items_offset = off;
    off += up256(sizeof(int32_t) * static_cast<size_t>(plan.groups.size()) * std::max(nbatch, 1));
  }
  const DeviceInfo info = device_info(dev);
  for (auto& g : plan.groups) {
    const bool mixed = o.form == TCHEM_GB_FORM_MIXED || o.form == TCHEM_GB_FORM_MIXED_SIMPLIFIED;
    if (mixed) g.dev = dts[g.mechs[0]]->dev_x;  // sliced-ELL tables
    const MechLayout& L = g.dev.L;
    plan.m_max = std::max(plan.m_max, L.m);
    g.form = o.form;
    if (mixed && L.m > 128 && !e3sm) {
      // beyond the register-resident shapes: the tensor-core full-Newton form, one sample per CTA
      if (L.m > tc_advance_max_species())
        throw std::domain_error("mixed forms: mechanisms with more than " + std::to_string(tc_advance_max_species()) +
                                " active species run in the plain form only");
      if (o.threads_per_sample != 0 && o.threads_per_sample != 128)
        throw std::domain_error("tensor-core form (more than 128 species): threads_per_sample must be 0 or 128");
      g.tc = true;
      g.dev = dts[g.mechs[0]]->dev;  // CSR tables, read from global memory
      g.form = o.form;
      g.threads_per_sample = 128;
      g.warps_per_block = 4;
      g.smem = tc_advance_smem_bytes(L);
      if (g.smem > static_cast<size_t>(info.max_smem_optin))
        throw std::domain_error("tensor-core form: working set larger than shared memory");
      g.grid = std::max(1, std::min(info.sm_count, std::max(nbatch, 1)));
      g.matrix_in_smem = false;
      g.lda = 0;
      g.gmat_elems_per_warp = tc_advance_matrix_floats();  // floats per CTA
      g.gmat_offset = off;
      off += up256(sizeof(float) * g.gmat_elems_per_warp * static_cast<size_t>(g.grid));
      continue;
    }
    if (mixed) {
      int tps = o.threads_per_sample;
      if (tps == 0 && o.form >= 0 && o.form < 3) tps = mechs[g.mechs[0]]->tps_pref[o.form];
      MixedConfig mc = mixed_config(L, tps, info.sm_count, info.max_smem_optin, nbatch,
                                    o.form == TCHEM_GB_FORM_MIXED_SIMPLIFIED, e3sm,
                                    g.dev.lu_prog ? g.dev.lu.nnz : 0);
      g.kernel = mc.kernel;
      g.warps_per_block = mc.warps_per_block;
      g.grid = mc.grid;
      g.smem = mc.smem;
      g.threads_per_sample = mc.threads_per_sample;
      g.ml = mc.ml;
      g.matrix_in_smem = true;
      g.lda = L.m;
      continue;
    }
    g.lda = L.m | 1;
    size_t ws = fp64_warp_smem_bytes(L, g.lda, true, e3sm);
    const size_t avail = static_cast<size_t>(info.max_smem_optin) - 16 - L.blob_bytes;
    int W = static_cast<int>(std::min<size_t>(kMaxWarpsPerBlock, avail / ws));
    if (W < 1) {
      g.matrix_in_smem = false;
      ws = fp64_warp_smem_bytes(L, g.lda, false, e3sm);
      W = static_cast<int>(std::min<size_t>(kMaxWarpsPerBlock, avail / ws));
      if (W < 1) throw std::invalid_argument("mechanism too large for the shared-memory working set");
    }
    g.warp_smem = static_cast<uint32_t>(ws);
    g.warps_per_block = W;
    g.smem = 16 + L.blob_bytes + static_cast<size_t>(W) * ws;
    g.kernel = trbdf2_fp64_kernel_ptr(L.m);
    cudaFuncSetAttribute(g.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(g.smem));
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, g.kernel, W * 32, g.smem) != cudaSuccess || bps < 1) bps = 1;
    const int need = (std::max(nbatch, 1) + W - 1) / W;
    g.grid = std::max(1, std::min(info.sm_count * bps, need));
    if (!g.matrix_in_smem) {
      g.gmat_elems_per_warp = static_cast<size_t>(L.m) * g.lda;
      g.gmat_offset = off;
      off += up256(sizeof(double) * g.gmat_elems_per_warp * static_cast<size_t>(g.grid) * W);
    }
  }
  plan.bytes = off;
  return plan;
}



tchem_gb_advance_opts opts_or_default(const tchem_gb_advance_opts* opts) {
  tchem_gb_advance_opts o{};
  if (opts) o = *opts;
  return o;
}

void fill_slots(const GroupPlan& g, const tchem_gb_mech* const* mechs, int dev, int n_mechs,
                const double* (&rate_param)[kMaxGroupSlots], int32_t (&slot_of_mech)[kMaxMechs]) {
  for (int i = 0; i < kMaxGroupSlots; ++i) rate_param[i] = nullptr;
  for (int i = 0; i < kMaxMechs; ++i) slot_of_mech[i] = -1;
  for (size_t s = 0; s < g.mechs.size(); ++s) {
    const int gm = g.mechs[s];
    rate_param[s] = mechs[gm]->device_tables[dev]->dev.rate_param;
    if (gm < n_mechs) slot_of_mech[gm] = static_cast<int32_t>(s);
  }
}

}  // namespace

int workspace_bytes_checked(const tchem_gb_mech* const* mechs, int n_mechs, int nbatch,
                            const tchem_gb_advance_opts* opts, size_t* bytes) {
  *bytes = 0;
  try {
    int dev = 0;
    cudaGetDevice(&dev);
    *bytes = make_plan(mechs, n_mechs, nbatch, n_mechs > 1, opts_or_default(opts), dev).bytes;
    return TCHEM_GB_OK;
  } catch (const std::domain_error& e) {
    return fail(TCHEM_GB_ERR_UNSUPPORTED, e.what());
  } catch (const std::bad_alloc&) {
    return fail(TCHEM_GB_ERR_NOMEM, "tchem_gb_workspace_bytes: allocation failed");
  } catch (const std::exception& e) {
    return fail(TCHEM_GB_ERR_ARG, e.what());
  }
}

}  // namespace tchem_gb

using namespace tchem_gb;

extern "C" {

size_t tchem_gb_workspace_bytes(const tchem_gb_mech* const* mechs, int n_mechs, int nbatch,
                                const tchem_gb_advance_opts* opts) {
  size_t bytes = 0;
  if (workspace_bytes_checked(mechs, n_mechs, nbatch, opts, &bytes) != TCHEM_GB_OK) return 0;
  int dev = 0;
  cudaGetDevice(&dev);
  noalloc_setup(dev);  // set-up time: load the fixed scratch of tchem_gb_time_advance_noalloc
  return bytes;
}

}  // extern "C"

namespace tchem_gb {
namespace {

// Trajectory-record arguments of the plain form (all null: no record).
struct TapeArgs {
  double* dt = nullptr;
  double* ckpt = nullptr;
  int32_t* nsteps = nullptr;
  int cap = 0;
  const double* k_scale = nullptr;
};

// E3SM inputs of the time-advance kernels (all null: the mechanism's rates and emissions).
struct RateArgs {
  const double* keff = nullptr;  // [B][R]
  const double* src = nullptr;   // source rows, row s at src + s * src_stride
  int64_t src_stride = 0;
};

int time_advance_impl(const tchem_gb_mech* const* mechs, int n_mechs, const int32_t* mech_of_sample, int nbatch,
                      const double* tol_newton, const double* tol_time, const tchem_gb_tadv* tadv,
                      const double* state, double* t_out, double* dt_out, double* state_out, int32_t* status,
                      tchem_gb_sample_stats* stats, void* workspace, size_t workspace_bytes,
                      const tchem_gb_advance_opts* opts, void* stream_v, const TapeArgs& tape,
                      const RateArgs& rates = RateArgs{}) {
  if (!mechs || nbatch < 0) return fail(TCHEM_GB_ERR_ARG, "tchem_gb_time_advance: bad mechanisms or batch size");
  if (nbatch == 0) return TCHEM_GB_OK;  // empty arrays may come with null pointers
  if (!tol_newton || !tol_time || !tadv || !state || !t_out || !dt_out || !state_out || !status)
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_time_advance: null argument");
  const tchem_gb_advance_opts o = opts_or_default(opts);
  if (o.form != TCHEM_GB_FORM_PLAIN_FP64 && o.form != TCHEM_GB_FORM_MIXED && o.form != TCHEM_GB_FORM_MIXED_SIMPLIFIED)
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_time_advance: unknown form");
  cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
  int dev = 0;
  cudaGetDevice(&dev);
  Plan plan;
  try {
    plan = make_plan(mechs, n_mechs, nbatch, mech_of_sample != nullptr, o, dev, rates.keff != nullptr);
    const int n0 = mechs[0]->km.nSpec;
    for (int i = 1; i < n_mechs; ++i)
      if (mechs[i]->km.nSpec + 3 > n0 + 3 && mech_of_sample == nullptr)
        throw std::invalid_argument("mechanisms of different sizes need mech_of_sample");
  } catch (const std::domain_error& e) {
    return fail(TCHEM_GB_ERR_UNSUPPORTED, e.what());
  } catch (const std::bad_alloc&) {
    return fail(TCHEM_GB_ERR_NOMEM, "tchem_gb_time_advance: allocation failed");
  } catch (const std::exception& e) {
    return fail(TCHEM_GB_ERR_ARG, e.what());
  }
  // All samples share one state row width: the widest mechanism's nSpec + 3.
  int state_dim = 0;
  for (int i = 0; i < n_mechs; ++i) state_dim = std::max(state_dim, mechs[i]->km.nSpec + 3);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  if (!ws) {
    try {
      ws = static_cast<unsigned char*>(owned_workspace(dev, plan.bytes));
    } catch (...) {
      return fail(TCHEM_GB_ERR_NOMEM, "tchem_gb_time_advance: workspace allocation failed");
    }
  } else if (workspace_bytes < plan.bytes) {
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_time_advance: workspace smaller than tchem_gb_workspace_bytes()");
  }
  int32_t* queue = reinterpret_cast<int32_t*>(ws);
  int32_t* error_word = reinterpret_cast<int32_t*>(ws + 64);
  int32_t* counts = reinterpret_cast<int32_t*>(ws + 128);
  cudaError_t e = cudaMemsetAsync(ws, 0, 64, stream);  // queues (the error word persists until read)
  if (e == cudaSuccess) e = cudaMemsetAsync(ws + 128, 0, 64, stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(workspace)");
  int32_t* items = plan.need_items ? reinterpret_cast<int32_t*>(ws + plan.items_offset) : nullptr;
  if (plan.need_items) {
    GroupMap G{};
    for (int i = 0; i < kMaxMechs; ++i) G.group_of_mech[i] = 0;
    for (size_t g = 0; g < plan.groups.size(); ++g)
      for (int gm : plan.groups[g].mechs) G.group_of_mech[gm] = static_cast<int32_t>(g);
    e = launch_bucket(mech_of_sample, nbatch, G, n_mechs, counts, items, status, stream);
    if (e != cudaSuccess) return cuda_fail(e, "bucket kernel");
    note_launch();
  }
  // Groups of different mechanism structures run concurrently: the largest mechanism's kernel is
  // launched first on the caller's stream, the others on side streams forked from it, so the
  // SMs that the first kernel's persistent CTAs release as its queue drains take the next
  // kernel's CTAs (no idle tail between kernels); the caller's stream joins them all.
  std::vector<size_t> order(plan.groups.size());
  for (size_t g = 0; g < order.size(); ++g) order[g] = g;
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t a, size_t b) { return plan.groups[a].dev.L.m > plan.groups[b].dev.L.m; });
  SideStreams* side = nullptr;
  std::unique_lock<std::mutex> side_lock;  // one caller at a time enqueues on the shared side streams
  if (plan.groups.size() > 1) {
    side = side_streams(dev);
    if (!side) return fail(TCHEM_GB_ERR_CUDA, "tchem_gb_time_advance: side stream creation failed");
    side_lock = std::unique_lock<std::mutex>(side->mu);
    e = cudaEventRecord(side->fork, stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventRecord(fork)");
  }
  for (size_t oi = 0; oi < order.size(); ++oi) {
    const size_t g = order[oi];
    const GroupPlan& gp = plan.groups[g];
    cudaStream_t gs = stream;
    if (oi > 0) {
      gs = side->s[oi - 1];
      e = cudaStreamWaitEvent(gs, side->fork, 0);
      if (e != cudaSuccess) return cuda_fail(e, "cudaStreamWaitEvent(fork)");
    }
    AdvanceParams P{};
    P.mech = gp.dev;
    fill_slots(gp, mechs, dev, n_mechs, P.rate_param, P.slot_of_mech);
    if (!mech_of_sample) {
      for (int i = 0; i < kMaxMechs; ++i) P.slot_of_mech[i] = -1;
      P.slot_of_mech[0] = 0;
    }
    P.mech_of_sample = mech_of_sample;
    P.items = plan.need_items ? items + g * static_cast<size_t>(nbatch) : nullptr;
    P.n_items_dev = plan.need_items ? counts + g : nullptr;
    P.n_items = nbatch;
    P.queue = queue + g;
    P.tol_newton = tol_newton;
    P.tol_time = tol_time;
    P.tadv = tadv;
    P.state = state;
    P.state_out = state_out;
    P.t_out = t_out;
    P.dt_out = dt_out;
    P.status = status;
    P.stats = stats;
    P.state_dim = state_dim;
    P.gmat = gp.matrix_in_smem ? nullptr : reinterpret_cast<double*>(ws + gp.gmat_offset);
    P.gmat_stride = static_cast<int64_t>(gp.gmat_elems_per_warp);
    P.lda = gp.lda;
    P.matrix_in_smem = gp.matrix_in_smem ? 1 : 0;
    P.warp_smem_bytes = gp.warp_smem;
    P.error_word = error_word;
    P.ml = gp.ml;
    P.tape_dt = tape.dt;
    P.tape_ckpt = tape.ckpt;
    P.tape_nsteps = tape.nsteps;
    P.tape_cap = tape.cap;
    P.k_scale = tape.k_scale;
    P.keff_in = rates.keff;
    P.src_in = rates.src;
    P.src_stride = rates.src_stride;
    if (gp.tc)
      e = launch_trbdf2_tc(P, gp.grid, gp.smem, gs);
    else if (gp.form == TCHEM_GB_FORM_MIXED || gp.form == TCHEM_GB_FORM_MIXED_SIMPLIFIED)
      e = launch_trbdf2_mixed(P, gp.dev.L, gp.grid, gp.warps_per_block, gp.smem, gp.threads_per_sample, gs);
    else
      e = launch_trbdf2_fp64(P, gp.grid, gp.warps_per_block, gp.smem, gs);
    if (e != cudaSuccess) return cuda_fail(e, "time-advance kernel launch");
    note_launch();
    if (oi > 0) {
      e = cudaEventRecord(side->join[oi - 1], gs);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, side->join[oi - 1], 0);
      if (e != cudaSuccess) return cuda_fail(e, "stream join");
    }
  }
  return TCHEM_GB_OK;
}

}  // namespace
}  // namespace tchem_gb

extern "C" {

int tchem_gb_time_advance(const tchem_gb_mech* const* mechs, int n_mechs, const int32_t* mech_of_sample, int nbatch,
                          const double* tol_newton, const double* tol_time, const double* /*fac*/,
                          const tchem_gb_tadv* tadv, const double* state, double* t_out, double* dt_out,
                          double* state_out, int32_t* status, tchem_gb_sample_stats* stats, void* workspace,
                          size_t workspace_bytes, const tchem_gb_advance_opts* opts, void* stream_v) {
  ProfileRegion region(mech_of_sample ? "TChem::AtmosphericChemistry::runDeviceBatch::kmcd array"
                                      : "TChem::AtmosphericChemistry::runDeviceBatch::kmcd");
  return time_advance_impl(mechs, n_mechs, mech_of_sample, nbatch, tol_newton, tol_time, tadv, state, t_out, dt_out,
                           state_out, status, stats, workspace, workspace_bytes, opts, stream_v, TapeArgs{});
}

int tchem_gb_time_advance_record(const tchem_gb_mech* mech, int nbatch, const double* tol_newton,
                                 const double* tol_time, const double* k_scale, const tchem_gb_tadv* tadv,
                                 const double* state, double* t_out, double* dt_out, double* state_out,
                                 int32_t* status, tchem_gb_sample_stats* stats, double* tape_dt, double* tape_ckpt,
                                 int32_t* tape_nsteps, int tape_cap, void* stream) {
  if (!mech) return fail(TCHEM_GB_ERR_ARG, "tchem_gb_time_advance_record: null mechanism");
  if (nbatch > 0 && (!tape_dt || !tape_ckpt || !tape_nsteps || tape_cap < 1))
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_time_advance_record: null trajectory record or tape_cap < 1");
  TapeArgs tape;
  tape.dt = tape_dt;
  tape.ckpt = tape_ckpt;
  tape.nsteps = tape_nsteps;
  tape.cap = tape_cap;
  tape.k_scale = k_scale;
  tchem_gb_advance_opts o{};
  o.form = TCHEM_GB_FORM_PLAIN_FP64;
  const tchem_gb_mech* mechs[1] = {mech};
  return time_advance_impl(mechs, 1, nullptr, nbatch, tol_newton, tol_time, tadv, state, t_out, dt_out, state_out,
                           status, stats, nullptr, 0, &o, stream, tape);
}

}  // extern "C"

namespace tchem_gb {
namespace {

struct AdjointPlan {
  int warps = 0, grid = 0, lda = 0;
  bool matrix_in_smem = true;
  size_t smem = 0, warp_smem = 0;
  size_t seg_offset = 0, seg_stride = 0, gmat_offset = 0, gmat_stride = 0, bytes = 0;
};

AdjointPlan make_adjoint_plan(const MechLayout& L, int nbatch, int dev) {
  const DeviceInfo info = device_info(dev);
  AdjointPlan a;
  a.lda = L.m | 1;
  const size_t avail = static_cast<size_t>(info.max_smem_optin) - 16 - L.blob_bytes;
  size_t ws = adjoint_warp_smem_bytes(L, a.lda, true);
  if (ws > avail) {
    a.matrix_in_smem = false;
    ws = adjoint_warp_smem_bytes(L, a.lda, false);
    if (ws > avail) throw std::invalid_argument("mechanism too large for the adjoint's shared-memory working set");
  }
  a.warps = static_cast<int>(std::min<size_t>(kMaxWarpsPerBlock, avail / ws));
  a.warp_smem = ws;
  a.smem = 16 + L.blob_bytes + a.warps * ws;
  const void* k = adjoint_kernel_ptr(L.m);
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(a.smem));
  int bps = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, a.warps * 32, a.smem) != cudaSuccess || bps < 1) bps = 1;
  a.grid = std::max(1, std::min(info.sm_count * bps, (std::max(nbatch, 1) + a.warps - 1) / a.warps));
  const size_t nw = static_cast<size_t>(a.grid) * a.warps;
  size_t off = kHeaderBytes;
  a.seg_stride = static_cast<size_t>(2 * kTapeSegment) * L.m;
  a.seg_offset = off;
  off += up256(sizeof(double) * a.seg_stride * nw);
  if (!a.matrix_in_smem) {
    a.gmat_stride = static_cast<size_t>(L.m) * a.lda;
    a.gmat_offset = off;
    off += up256(sizeof(double) * a.gmat_stride * nw);
  }
  a.bytes = off;
  return a;
}

}  // namespace
}  // namespace tchem_gb

extern "C" {

size_t tchem_gb_adjoint_workspace_bytes(const tchem_gb_mech* mech, int nbatch) {
  try {
    if (!mech) throw std::invalid_argument("null mechanism");
    int dev = 0;
    cudaGetDevice(&dev);
    return make_adjoint_plan(tables_for(mech, dev)->dev.L, nbatch, dev).bytes;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return 0;
  }
}

int tchem_gb_adjoint(const tchem_gb_mech* mech, int nbatch, const double* tol_newton, const double* k_scale,
                     const tchem_gb_tadv* tadv, const double* state, const double* tape_dt, const double* tape_ckpt,
                     const int32_t* tape_nsteps, int tape_cap, const double* lambda, double* grad_x0, double* grad_k,
                     int32_t* status, void* workspace, size_t workspace_bytes, void* stream_v) {
  if (!mech || nbatch < 0) return fail(TCHEM_GB_ERR_ARG, "tchem_gb_adjoint: bad mechanism or batch size");
  if (nbatch == 0) return TCHEM_GB_OK;
  if (!tol_newton || !tadv || !state || !tape_dt || !tape_ckpt || !tape_nsteps || tape_cap < 1 || !lambda ||
      !grad_x0 || !grad_k || !status)
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_adjoint: null argument or tape_cap < 1");
  int dev = 0;
  cudaGetDevice(&dev);
  cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
  AdjointParams P{};
  AdjointPlan a;
  try {
    const DeviceTables* t = tables_for(mech, dev);
    if (!mech->host_tables->supported) throw std::domain_error(mech->host_tables->unsupported_reason);
    a = make_adjoint_plan(t->dev.L, nbatch, dev);
    P.mech = t->dev;
    P.rate_param = t->dev.rate_param;
  } catch (const std::domain_error& e) {
    return fail(TCHEM_GB_ERR_UNSUPPORTED, e.what());
  } catch (const std::exception& e) {
    return fail(TCHEM_GB_ERR_ARG, e.what());
  }
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  if (!ws) {
    try {
      ws = static_cast<unsigned char*>(owned_workspace(dev, a.bytes));
    } catch (...) {
      return fail(TCHEM_GB_ERR_NOMEM, "tchem_gb_adjoint: workspace allocation failed");
    }
  } else if (workspace_bytes < a.bytes) {
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_adjoint: workspace smaller than tchem_gb_adjoint_workspace_bytes()");
  }
  cudaError_t e = cudaMemsetAsync(ws, 0, 64, stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(workspace)");
  P.k_scale = k_scale;
  P.B = nbatch;
  P.state = state;
  P.state_dim = mech->km.nSpec + 3;
  P.tadv = tadv;
  P.tol_newton = tol_newton;
  P.tape_dt = tape_dt;
  P.tape_ckpt = tape_ckpt;
  P.tape_nsteps = tape_nsteps;
  P.tape_cap = tape_cap;
  P.lambda = lambda;
  P.grad_x0 = grad_x0;
  P.grad_k = grad_k;
  P.status = status;
  P.seg = reinterpret_cast<double*>(ws + a.seg_offset);
  P.seg_stride = static_cast<int64_t>(a.seg_stride);
  P.gmat = a.matrix_in_smem ? nullptr : reinterpret_cast<double*>(ws + a.gmat_offset);
  P.gmat_stride = static_cast<int64_t>(a.gmat_stride);
  P.lda = a.lda;
  P.matrix_in_smem = a.matrix_in_smem ? 1 : 0;
  P.warp_smem_bytes = static_cast<uint32_t>(a.warp_smem);
  P.queue = reinterpret_cast<int32_t*>(ws);
  P.error_word = reinterpret_cast<int32_t*>(ws + 64);
  e = launch_adjoint(P, a.grid, a.warps, a.smem, stream);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint kernel launch");
  note_launch();
  return TCHEM_GB_OK;
}

int tchem_gb_mech_set_threads_per_sample(tchem_gb_mech* mech, int form, int threads_per_sample) {
  if (!mech || form < 0 || form > 2 ||
      (threads_per_sample != 0 && threads_per_sample != 32 && threads_per_sample != 64 && threads_per_sample != 128))
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_mech_set_threads_per_sample: bad argument");
  std::lock_guard<std::mutex> lk(mech->mu);
  mech->tps_pref[form] = threads_per_sample;
  return TCHEM_GB_OK;
}

int tchem_gb_autotune(tchem_gb_mech* mech, int form, int nbatch, const double* tol_newton, const double* tol_time,
                      const tchem_gb_tadv* tadv, const double* state, double* t_out, double* dt_out,
                      double* state_out, int32_t* status, void* workspace, size_t workspace_bytes, void* stream_v,
                      int* chosen, float* ms_per_candidate) {
  if (!mech || form < 0 || form > 2 || nbatch <= 0 || !chosen)
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_autotune: bad argument");
  const int cands[3] = {32, 64, 128};
  cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return fail(TCHEM_GB_ERR_CUDA, "tchem_gb_autotune: cudaEventCreate failed");
  float best_ms = 0.f;
  int best = 0;
  const tchem_gb_mech* mechs[1] = {mech};
  for (int c = 0; c < 3; ++c) {
    if (ms_per_candidate) ms_per_candidate[c] = -1.f;
    tchem_gb_advance_opts o{};
    o.form = form;
    o.threads_per_sample = cands[c];
    if (form == TCHEM_GB_FORM_PLAIN_FP64 && cands[c] != 32) continue;  // the plain form has one shape
    if (tchem_gb_workspace_bytes(mechs, 1, nbatch, &o) == 0) continue;  // no kernel of this shape
    cudaMemsetAsync(t_out, 0, sizeof(double) * nbatch, stream);       // the probe starts at t = 0
    cudaEventRecord(e0, stream);
    const int rc = time_advance_impl(mechs, 1, nullptr, nbatch, tol_newton, tol_time, tadv, state, t_out, dt_out,
                                     state_out, status, nullptr, workspace, workspace_bytes, &o, stream_v, TapeArgs{});
    cudaEventRecord(e1, stream);
    if (rc != TCHEM_GB_OK) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return rc;
    }
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return fail(TCHEM_GB_ERR_CUDA, "tchem_gb_autotune: probe run failed");
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms_per_candidate) ms_per_candidate[c] = ms;
    if (best == 0 || ms < best_ms) {
      best = cands[c];
      best_ms = ms;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best == 0) return fail(TCHEM_GB_ERR_UNSUPPORTED, "tchem_gb_autotune: no kernel shape for this mechanism");
  {
    std::lock_guard<std::mutex> lk(mech->mu);
    mech->tps_pref[form] = best;
  }
  *chosen = best;
  return TCHEM_GB_OK;
}

long long tchem_gb_kernel_launches(void) { return g_kernel_launches.load(std::memory_order_relaxed); }

int tchem_gb_device_error(void* workspace, void* stream_v, int32_t* device_error) {
  if (!device_error) return fail(TCHEM_GB_ERR_ARG, "tchem_gb_device_error: null argument");
  cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  int dev = 0;
  cudaGetDevice(&dev);
  unsigned char* ws = static_cast<unsigned char*>(workspace ? workspace : owned_workspace_peek(dev));
  *device_error = 0;
  if (!ws) return TCHEM_GB_OK;
  e = cudaMemcpy(device_error, ws + 64, sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(ws + 64, 0, sizeof(int32_t));
  if (e != cudaSuccess) return cuda_fail(e, "tchem_gb_device_error");
  return TCHEM_GB_OK;
}

namespace {

struct HostBufCache {
  void* ptr = nullptr;
  size_t bytes = 0;
};
std::mutex g_hb_mu;
std::vector<HostBufCache> g_hb;

int run_unit(const tchem_gb_mech* const* mechs, int n_mechs, const int32_t* mech_of_sample, int nbatch,
             const double* state, double* out, void* stream_v, UnitKind kind) {
  if (!mechs || n_mechs <= 0 || n_mechs > kMaxGroupSlots || nbatch < 0)
    return fail(TCHEM_GB_ERR_ARG, "unit entry point: bad argument");
  if (nbatch == 0) return TCHEM_GB_OK;
  if (!state || !out) return fail(TCHEM_GB_ERR_ARG, "unit entry point: null array");
  int dev = 0;
  cudaGetDevice(&dev);
  UnitParams P{};
  try {
    const DeviceTables* t0 = tables_for(mechs[0], dev);
    const HostTables* h0 = mechs[0]->host_tables.get();
    if (!h0->supported && kind != UNIT_KFORWARD) throw std::domain_error(h0->unsupported_reason);
    P.mech = t0->dev;
    for (int i = 0; i < kMaxMechs; ++i) P.slot_of_mech[i] = -1;
    for (int i = 0; i < n_mechs; ++i) {
      const DeviceTables* ti = tables_for(mechs[i], dev);
      if (mechs[i]->host_tables->signature != h0->signature)
        throw std::invalid_argument("unit entry points need mechanisms of one structure");
      P.rate_param[i] = ti->dev.rate_param;
      P.slot_of_mech[i] = i;
    }
  } catch (const std::domain_error& e) {
    return fail(TCHEM_GB_ERR_UNSUPPORTED, e.what());
  } catch (const std::exception& e) {
    return fail(TCHEM_GB_ERR_ARG, e.what());
  }
  unsigned char* ws = nullptr;
  try {
    ws = static_cast<unsigned char*>(owned_workspace(dev, kHeaderBytes));
  } catch (...) {
    return fail(TCHEM_GB_ERR_NOMEM, "workspace allocation failed");
  }
  P.mech_of_sample = mech_of_sample;
  P.B = nbatch;
  P.state = state;
  P.state_dim = mechs[0]->km.nSpec + 3;
  P.out = out;
  P.error_word = reinterpret_cast<int32_t*>(ws + 64);
  P.status = nullptr;
  cudaError_t e = launch_unit(P, kind, static_cast<cudaStream_t>(stream_v));
  if (e != cudaSuccess) return cuda_fail(e, "unit kernel launch");
  note_launch();
  return TCHEM_GB_OK;
}

}  // namespace

int tchem_gb_kforward(const tchem_gb_mech* const* mechs, int n_mechs, const int32_t* mech_of_sample, int nbatch,
                      const double* state, double* kfor, void* stream) {
  return run_unit(mechs, n_mechs, mech_of_sample, nbatch, state, kfor, stream, UNIT_KFORWARD);
}

int tchem_gb_reaction_rates(const tchem_gb_mech* const* mechs, int n_mechs, const int32_t* mech_of_sample,
                            int nbatch, const double* state, double* omega, void* stream) {
  return run_unit(mechs, n_mechs, mech_of_sample, nbatch, state, omega, stream, UNIT_RHS);
}

int tchem_gb_jacobian(const tchem_gb_mech* const* mechs, int n_mechs, const int32_t* mech_of_sample, int nbatch,
                      const double* state, double* jac, void* stream) {
  return run_unit(mechs, n_mechs, mech_of_sample, nbatch, state, jac, stream, UNIT_JACOBIAN);
}

int tchem_gb_time_advance_hostbuf(const tchem_gb_mech* const* mechs, int n_mechs, const int32_t* mech_of_sample,
                                  int nbatch, const double* tol_newton, const double* tol_time,
                                  const tchem_gb_tadv* tadv, const double* state, double* t_out,
                                  double* dt_out, double* state_out, int32_t* status, tchem_gb_sample_stats* stats,
                                  const tchem_gb_advance_opts* opts, void* stream_v) {
  ProfileRegion region(mech_of_sample ? "TChem::AtmosphericChemistry::runHostBatch::kmcd array"
                                      : "TChem::AtmosphericChemistry::runHostBatch::kmcd");
  if (!mechs || n_mechs <= 0 || nbatch < 0)
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_time_advance_hostbuf: bad mechanisms or batch size");
  if (nbatch == 0) return TCHEM_GB_OK;
  if (!tol_newton || !tol_time || !tadv || !state || !t_out || !dt_out || !state_out || !status)
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_time_advance_hostbuf: null argument");
  cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
  int dev = 0;
  cudaGetDevice(&dev);
  int m_max = 0, dim = 0;
  for (int i = 0; i < n_mechs; ++i) {
    if (!mechs[i]) return fail(TCHEM_GB_ERR_ARG, "null mechanism handle");
    m_max = std::max(m_max, mechs[i]->km.nActive());
    dim = std::max(dim, mechs[i]->km.nSpec + 3);
  }
  const size_t B = static_cast<size_t>(nbatch);
  size_t off = 0;
  auto sec = [&](size_t bytes) { const size_t o = off; off += up256(bytes); return o; };
  const size_t o_tn = sec(2 * sizeof(double));
  const size_t o_tt = sec(2 * sizeof(double) * m_max);
  const size_t o_tadv = sec(sizeof(tchem_gb_tadv) * B);
  const size_t o_state = sec(sizeof(double) * B * dim);
  const size_t o_sout = sec(sizeof(double) * B * dim);
  const size_t o_t = sec(sizeof(double) * B);
  const size_t o_dt = sec(sizeof(double) * B);
  const size_t o_st = sec(sizeof(int32_t) * B);
  const size_t o_stats = sec(sizeof(tchem_gb_sample_stats) * B);
  const size_t o_mos = sec(sizeof(int32_t) * B);
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_hb_mu);
    if (static_cast<int>(g_hb.size()) <= dev) g_hb.resize(dev + 1);
    HostBufCache& c = g_hb[dev];
    if (c.bytes < off) {
      if (c.ptr) {
        cudaDeviceSynchronize();
        cudaFree(c.ptr);
      }
      c.ptr = nullptr;
      c.bytes = 0;
      if (cudaMalloc(&c.ptr, off) != cudaSuccess) {
        cudaGetLastError();
        return fail(TCHEM_GB_ERR_NOMEM, "tchem_gb_time_advance_hostbuf: device buffer allocation failed");
      }
      c.bytes = off;
    }
    base = static_cast<unsigned char*>(c.ptr);
  }
  auto h2d = [&](size_t o, const void* src, size_t bytes) {
    return cudaMemcpyAsync(base + o, src, bytes, cudaMemcpyHostToDevice, stream);
  };
  cudaError_t e = h2d(o_tn, tol_newton, 2 * sizeof(double));
  if (e == cudaSuccess) e = h2d(o_tt, tol_time, 2 * sizeof(double) * m_max);
  if (e == cudaSuccess) e = h2d(o_tadv, tadv, sizeof(tchem_gb_tadv) * B);
  if (e == cudaSuccess) e = h2d(o_state, state, sizeof(double) * B * dim);
  if (e == cudaSuccess) e = h2d(o_t, t_out, sizeof(double) * B);
  if (e == cudaSuccess && mech_of_sample) e = h2d(o_mos, mech_of_sample, sizeof(int32_t) * B);
  if (e != cudaSuccess) return cuda_fail(e, "tchem_gb_time_advance_hostbuf: host-to-device copy");
  // state_out starts as a copy of state so rows of skipped samples come back unchanged.
  e = cudaMemcpyAsync(base + o_sout, base + o_state, sizeof(double) * B * dim, cudaMemcpyDeviceToDevice, stream);
  if (e != cudaSuccess) return cuda_fail(e, "tchem_gb_time_advance_hostbuf: device copy");
  const int rc = tchem_gb_time_advance(
      mechs, n_mechs, mech_of_sample ? reinterpret_cast<const int32_t*>(base + o_mos) : nullptr, nbatch,
      reinterpret_cast<const double*>(base + o_tn), reinterpret_cast<const double*>(base + o_tt), nullptr,
      reinterpret_cast<const tchem_gb_tadv*>(base + o_tadv), reinterpret_cast<const double*>(base + o_state),
      reinterpret_cast<double*>(base + o_t), reinterpret_cast<double*>(base + o_dt),
      reinterpret_cast<double*>(base + o_sout), reinterpret_cast<int32_t*>(base + o_st),
      stats ? reinterpret_cast<tchem_gb_sample_stats*>(base + o_stats) : nullptr, nullptr, 0, opts, stream_v);
  if (rc != TCHEM_GB_OK) return rc;
  auto d2h = [&](void* dst, size_t o, size_t bytes) {
    return cudaMemcpyAsync(dst, base + o, bytes, cudaMemcpyDeviceToHost, stream);
  };
  e = d2h(state_out, o_sout, sizeof(double) * B * dim);
  if (e == cudaSuccess) e = d2h(t_out, o_t, sizeof(double) * B);
  if (e == cudaSuccess) e = d2h(dt_out, o_dt, sizeof(double) * B);
  if (e == cudaSuccess) e = d2h(status, o_st, sizeof(int32_t) * B);
  if (e == cudaSuccess && stats) e = d2h(stats, o_stats, sizeof(tchem_gb_sample_stats) * B);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_fail(e, "tchem_gb_time_advance_hostbuf: device-to-host copy");
  return TCHEM_GB_OK;
}

}  // extern "C"

// ---- E3SM gas chemistry -----------------------------------------------------------------------

namespace tchem_gb {
namespace {

// Tables of one mechanism for the E3SM kernels (throws domain_error when they cannot drive them).
const DeviceTables* e3sm_tables(const tchem_gb_mech* mech, int dev) {
  if (!mech) throw std::invalid_argument("null mechanism");
  const DeviceTables* t = tables_for(mech, dev);
  if (!mech->host_tables->e3sm_valid) throw std::domain_error(mech->host_tables->e3sm_invalid_reason);
  return t;
}

int run_e3sm_rates(const tchem_gb_mech* mech, int nbatch, const double* state, const double* photo_rates, int n_photo,
                   const double* external_sources, double* out, void* stream_v, E3smOut kind, const char* who) {
  if (!mech || nbatch < 0 || n_photo < 0 || (n_photo > 0 && !photo_rates))
    return fail(TCHEM_GB_ERR_ARG, std::string(who) + ": bad argument");
  if (nbatch == 0) return TCHEM_GB_OK;
  if (!state || !out) return fail(TCHEM_GB_ERR_ARG, std::string(who) + ": null array");
  int dev = 0;
  cudaGetDevice(&dev);
  E3smParams P{};
  try {
    P.mech = e3sm_tables(mech, dev)->dev;
  } catch (const std::domain_error& e) {
    return fail(TCHEM_GB_ERR_UNSUPPORTED, e.what());
  } catch (const std::exception& e) {
    return fail(TCHEM_GB_ERR_ARG, e.what());
  }
  P.B = nbatch;
  P.state = state;
  P.state_dim = mech->km.nSpec + 3;
  P.photo = n_photo > 0 ? photo_rates : nullptr;
  P.n_photo = n_photo;
  P.ext = external_sources;
  P.out = out;
  const cudaError_t e = launch_e3sm(P, kind, device_info(dev).sm_count, static_cast<cudaStream_t>(stream_v));
  if (e != cudaSuccess) return cuda_fail(e, who);
  note_launch();
  return TCHEM_GB_OK;
}

// Workspace of the E3SM time advance: the time-advance plan, then keff[B][R], then one zero row of
// m source terms (used when the caller passes no external sources).
struct E3smLayout {
  size_t plan_bytes = 0, keff_offset = 0, zero_offset = 0, bytes = 0;
};

E3smLayout e3sm_layout(const tchem_gb_mech* mech, int nbatch, const tchem_gb_advance_opts& o, int dev) {
  e3sm_tables(mech, dev);
  const tchem_gb_mech* mechs[1] = {mech};
  E3smLayout l;
  l.plan_bytes = make_plan(mechs, 1, nbatch, false, o, dev, true).bytes;
  l.keff_offset = up256(l.plan_bytes);
  l.zero_offset = l.keff_offset + up256(sizeof(double) * static_cast<size_t>(std::max(nbatch, 1)) * mech->km.nReac);
  l.bytes = l.zero_offset + up256(sizeof(double) * mech->km.nActive());
  return l;
}

}  // namespace
}  // namespace tchem_gb

extern "C" {

int tchem_gb_e3sm_reaction_rates(const tchem_gb_mech* mech, int nbatch, const double* state,
                                 const double* photo_rates, int n_photo, double* kfor, void* stream) {
  return run_e3sm_rates(mech, nbatch, state, photo_rates, n_photo, nullptr, kfor, stream, E3SM_KFOR,
                        "tchem_gb_e3sm_reaction_rates");
}

int tchem_gb_e3sm_rate_of_progress(const tchem_gb_mech* mech, int nbatch, const double* state,
                                   const double* photo_rates, int n_photo, double* rop, void* stream) {
  return run_e3sm_rates(mech, nbatch, state, photo_rates, n_photo, nullptr, rop, stream, E3SM_ROP,
                        "tchem_gb_e3sm_rate_of_progress");
}

int tchem_gb_e3sm_net_production_rates(const tchem_gb_mech* mech, int nbatch, const double* state,
                                       const double* photo_rates, int n_photo, const double* external_sources,
                                       double* omega, void* stream) {
  return run_e3sm_rates(mech, nbatch, state, photo_rates, n_photo, external_sources, omega, stream, E3SM_OMEGA,
                        "tchem_gb_e3sm_net_production_rates");
}

size_t tchem_gb_e3sm_workspace_bytes(const tchem_gb_mech* mech, int nbatch, const tchem_gb_advance_opts* opts) {
  try {
    int dev = 0;
    cudaGetDevice(&dev);
    return e3sm_layout(mech, nbatch, opts_or_default(opts), dev).bytes;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return 0;
  }
}

int tchem_gb_e3sm_time_advance(const tchem_gb_mech* mech, int nbatch, const double* tol_newton,
                               const double* tol_time, const double* /*fac*/, const tchem_gb_tadv* tadv,
                               const double* state, const double* photo_rates, int n_photo,
                               const double* external_sources, double* t_out, double* dt_out, double* state_out,
                               int32_t* status, tchem_gb_sample_stats* stats, void* workspace,
                               size_t workspace_bytes, const tchem_gb_advance_opts* opts, void* stream_v) {
  ProfileRegion region("TChem::AtmosphericChemistryE3SM::runDeviceBatch::kmcd");
  if (!mech || nbatch < 0 || n_photo < 0 || (n_photo > 0 && !photo_rates))
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_e3sm_time_advance: bad argument");
  if (nbatch == 0) return TCHEM_GB_OK;
  if (!tol_newton || !tol_time || !tadv || !state || !t_out || !dt_out || !state_out || !status)
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_e3sm_time_advance: null argument");
  const tchem_gb_advance_opts o = opts_or_default(opts);
  if (o.form != TCHEM_GB_FORM_PLAIN_FP64 && o.form != TCHEM_GB_FORM_MIXED && o.form != TCHEM_GB_FORM_MIXED_SIMPLIFIED)
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_e3sm_time_advance: unknown form");
  int dev = 0;
  cudaGetDevice(&dev);
  E3smLayout l;
  try {
    l = e3sm_layout(mech, nbatch, o, dev);
  } catch (const std::domain_error& e) {
    return fail(TCHEM_GB_ERR_UNSUPPORTED, e.what());
  } catch (const std::bad_alloc&) {
    return fail(TCHEM_GB_ERR_NOMEM, "tchem_gb_e3sm_time_advance: allocation failed");
  } catch (const std::exception& e) {
    return fail(TCHEM_GB_ERR_ARG, e.what());
  }
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  if (!ws) {
    try {
      ws = static_cast<unsigned char*>(owned_workspace(dev, l.bytes));
    } catch (...) {
      return fail(TCHEM_GB_ERR_NOMEM, "tchem_gb_e3sm_time_advance: workspace allocation failed");
    }
    workspace_bytes = l.bytes;
  } else if (workspace_bytes < l.bytes) {
    return fail(TCHEM_GB_ERR_ARG, "tchem_gb_e3sm_time_advance: workspace smaller than tchem_gb_e3sm_workspace_bytes()");
  }
  cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
  double* keff = reinterpret_cast<double*>(ws + l.keff_offset);
  E3smParams E{};
  E.mech = mech->device_tables[dev]->dev;
  E.B = nbatch;
  E.state = state;
  E.state_dim = mech->km.nSpec + 3;
  E.photo = n_photo > 0 ? photo_rates : nullptr;
  E.n_photo = n_photo;
  E.out = keff;
  cudaError_t e = launch_e3sm(E, E3SM_KEFF, device_info(dev).sm_count, stream);
  if (e != cudaSuccess) return cuda_fail(e, "E3SM rate-constant kernel launch");
  note_launch();
  RateArgs ra;
  ra.keff = keff;
  if (external_sources) {
    ra.src = external_sources;
    ra.src_stride = mech->km.nActive();
  } else {
    ra.src = reinterpret_cast<const double*>(ws + l.zero_offset);
    ra.src_stride = 0;
    e = cudaMemsetAsync(ws + l.zero_offset, 0, sizeof(double) * mech->km.nActive(), stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(workspace)");
  }
  const tchem_gb_mech* mechs[1] = {mech};
  return time_advance_impl(mechs, 1, nullptr, nbatch, tol_newton, tol_time, tadv, state, t_out, dt_out, state_out,
                           status, stats, ws, workspace_bytes, &o, stream_v, TapeArgs{}, ra);
}

}  // extern "C"

// C-ABI of the GB300 ConicXX path (declared in include/conicxx_gb300.h).
//
// cxg_batch: N independent instances; one persistent launch per size bucket, instances taken
// heaviest-first from an atomic queue; the device-side sequence (queue resets + launches) is
// captured once into a CUDA graph and replayed on every solve.
// cxg_solver: conicxx::Solver semantics (include/conicxx/solver.h) over a batch of one, FP64
// factorisation by default (the plain per-instance GPU form).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <thread>
#include <type_traits>
#include <numeric>
#include <string>
#include <vector>

#include "conicxx_gb300.h"
#include "cxg_kernels.h"
#include "cxg_layout.h"
#include "cxg_plan.h"

using namespace cxg;

static thread_local std::string g_lastError;

namespace cxg {
std::string& lastErrorRef() { return g_lastError; }
}  // namespace cxg

static int setErr(int code, const std::string& msg) {
  g_lastError = msg;
  return code;
}

#define CX_CUDA(call)                                                                        \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return setErr(CXG_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));         \
  } while (0)

extern "C" const char* cxg_last_error(void) { return g_lastError.c_str(); }
extern "C" const char* cxg_version(void) { return "conicxx_gb300 0.1.0"; }

extern "C" int cxg_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

extern "C" const char* cxg_status_string(int status) {
  switch (status) {
    case CXG_STATUS_UNSOLVED: return "Unsolved";
    case CXG_STATUS_SOLVED: return "Solved";
    case CXG_STATUS_PRIMAL_INFEASIBLE: return "PrimalInfeasible";
    case CXG_STATUS_DUAL_INFEASIBLE: return "DualInfeasible";
    case CXG_STATUS_MAX_ITERATIONS: return "MaxIterations";
    case CXG_STATUS_NUMERICAL_ERROR: return "NumericalError";
  }
  return "Unknown";
}

extern "C" void cxg_default_settings(cxg_settings* s) {
  if (!s) return;
  std::memset(s, 0, sizeof(*s));
  s->tol_feas = 1e-8;
  s->tol_gap_abs = 1e-8;
  s->tol_gap_rel = 1e-8;
  s->tol_infeas = 1e-7;
  s->max_iter = 200;
  s->static_reg_P = 1e-8;
  s->static_reg_A = 1e-8;
  s->dynamic_reg_eps = 1e-14;
  s->dynamic_reg_delta = 1e-7;
  s->refine_max_iter = 3;
  s->refine_tol = 1e-12;
  s->max_step_fraction = 0.99;
  s->equilibrate = 1;
  s->equilibrate_max_iter = 10;
  s->equilibrate_min_scale = 1e-4;
  s->equilibrate_max_scale = 1e4;
  s->warm_start = 1;
  s->verbose = 0;
  s->record_timings = 0;
  s->validate_inputs = 1;
  s->linear_solver = CXG_LINSOLVER_QDLDL;
  s->precision = CXG_PRECISION_FP64;
  s->mixed_refine_max_iter = 4;
  s->mixed_fallback_tol = 1e-10;
  s->threads_per_instance = 0;
  s->differentiable = 0;
  s->whole_gpu_root = 0;
  s->fault_factor_failures = 0;
  s->fault_nonfinite_solves = 0;
  s->soc_reference_dense = 1;
}

// ------------------------------------------------------------------------------------------
// batch
// ------------------------------------------------------------------------------------------
struct Group {
  int begin = 0, count = 0;  // range in `order`
  int block = 128, grid = 1;
  bool fp32 = false;
  SmemLayout lay{};
  size_t smem = 0;
  int64_t stride = 0;        // scratch doubles per CTA
  int64_t scratchOff = 0;    // offset of this group's scratch in the batch scratch buffer
  int occupancy = 1;         // resident CTAs per SM of this bucket's launch shape
  int gridAlone = 1;         // persistent grid when the bucket runs alone (occupancy x SMs, capped by count)
  double work = 0.0;         // estimated SM time per iteration: sum over its instances of nr
  int counterIdx = 0;
};

struct cxg_batch {
  int count = 0;
  cxg_settings st{};      // current settings
  cxg_settings kktSt{};   // KKT fields frozen at setup (kkt_system.cpp:26-31)
  Pools pools;
  std::vector<Pools> inst;                        // each instance's own plan (offsets from 0), for cxg_batch_replace
  size_t ipoolCap = 0, dpoolCap = 0;              // device capacity of dIpool / dDpool (entries)
  std::vector<int> edges;                         // size-bucket upper edges on nr (empty: kBucketEdges)
  std::vector<std::vector<int>> Pp, Pi, Ap, Ai;  // patterns for updateData checks
  std::vector<int> order;
  std::vector<Group> groups;
  // device
  InstanceDesc* dDesc = nullptr;
  int* dIpool = nullptr;
  double* dDpool = nullptr;
  double *dPx = nullptr, *dq = nullptr, *dAx = nullptr, *db = nullptr;
  double *dx = nullptr, *ds = nullptr, *dz = nullptr;
  DevResult* dRes = nullptr;
  double *dWx = nullptr, *dWs = nullptr, *dWz = nullptr;
  unsigned char* dHaveWarm = nullptr;
  double* dScratch = nullptr;
  double* dBwd = nullptr;                 // saved final states (differentiable)
  double *dGx = nullptr, *dGq = nullptr, *dGb = nullptr, *dGP = nullptr, *dGA = nullptr;
  int64_t bwdTotal = 0;
  int* dCounters = nullptr;
  int* dOrder = nullptr;
  cudaStream_t stream = nullptr;
  std::vector<cudaStream_t> groupStreams;   // one per size bucket (forked inside the graph)
  std::vector<cudaEvent_t> forkJoin;        // fork event + one join event per bucket
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graphExec = nullptr;
  DevSettings graphSettings{};
  bool graphValid = false;
  int64_t scratchCapacity = 0;              // doubles allocated in dScratch
  std::vector<DevResult> hRes;
  int lastLaunches = 0;
  double setupTime = 0.0;
  int device = 0;
  bool gridMode = false;                    // one instance, root spread over every SM (launchIpmGrid)
  bool bwdDropped = false;                  // differentiable asked for, not kept (whole-GPU root > 8192 rows)
  bool bwdStale = false;                    // instances replaced since the last solve: no saved states
  void* dGridCtl = nullptr;                 // its control block
  double* dTrace = nullptr;                 // record_timings: iteration traces (count x traceRows rows)
  int traceRows = 0;

  ~cxg_batch() {
    if (graphExec) cudaGraphExecDestroy(graphExec);
    if (graph) cudaGraphDestroy(graph);
    void* ptrs[] = {dDesc, dIpool, dDpool, dPx, dq, dAx, db, dx, ds, dz, dRes, dWx, dWs, dWz, dHaveWarm, dScratch,
                    dCounters, dOrder, dBwd, dGx, dGq, dGb, dGP, dGA, dGridCtl, dTrace};
    for (void* p : ptrs)
      if (p) cudaFree(p);
    for (cudaEvent_t e : forkJoin) cudaEventDestroy(e);
    for (cudaStream_t gs : groupStreams) cudaStreamDestroy(gs);
    if (stream) cudaStreamDestroy(stream);
  }
};

static DevSettings makeDevSettings(const cxg_settings& st, const cxg_settings& kk) {
  DevSettings d{};
  d.tol_feas = st.tol_feas;
  d.tol_gap_abs = st.tol_gap_abs;
  d.tol_gap_rel = st.tol_gap_rel;
  d.tol_infeas = st.tol_infeas;
  d.static_reg_P = kk.static_reg_P;
  d.static_reg_A = kk.static_reg_A;
  d.dynamic_reg_eps = kk.dynamic_reg_eps;
  d.dynamic_reg_delta = kk.dynamic_reg_delta;
  d.refine_tol = kk.refine_tol;
  d.max_step_fraction = st.max_step_fraction;
  d.mixed_fallback_tol = st.mixed_fallback_tol;
  d.max_iter = st.max_iter;
  d.refine_max_iter = kk.refine_max_iter;
  d.mixed_refine_max_iter = std::max(st.mixed_refine_max_iter, 0);
  d.linear_solver = kk.linear_solver;
  d.equilibrate = kk.equilibrate;
  d.warm_start = st.warm_start;
  d.precision = st.precision;
  d.record_timings = st.record_timings ? 1 : 0;
  d.fault_factor_failures = std::max(st.fault_factor_failures, 0);
  d.fault_nonfinite_solves = std::max(st.fault_nonfinite_solves, 0);
  d.soc_ref_dense = kk.soc_reference_dense ? 1 : 0;
  return d;
}

static bool sameDev(const DevSettings& a, const DevSettings& b) { return std::memcmp(&a, &b, sizeof(a)) == 0; }

template <typename T>
static int devAlloc(T** p, size_t count) {
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) return setErr(CXG_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return CXG_OK;
}

static int64_t r2(int64_t v) { return (v + 1) & ~int64_t(1); }

// Group boundaries on the root dimension nr; each group gets a shared-memory layout sized for
// its largest instance.
// Roots above 128 rows run 256-thread CTAs, one per SM, so the 128-192 range is one bucket: one
// history-ordered queue then starts all of its slowest instances first.
static const int kBucketEdges[] = {32, 64, 96, 128, 192, 256, 384, 512, 1024, 2048, 4096};
// Root sizes: the largest one-CTA root; cxg_solver spreads roots above kGridAutoRoot rows over
// every SM (whole_gpu_root = 0), which accepts up to kGridMaxRoot rows. The plan's root scatter
// maps hold 64-bit element offsets; a 131072-row root is 8.86e9 entries (71 GB of 8-byte
// entries), and the host planner and tile indices stay within 32 bits up to there.
static const int kCtaMaxRoot = 4096;
static const int kGridAutoRoot = 512;
static const int kGridMaxRoot = 131072;
static const int kGridMaxAdjointRoot = 8192;
// shared memory of the whole-GPU trailing update (8-byte entries; see gridStageBytes)
// (8-byte entries; see gridStageBytes), or the FP32 tensor-core update's, whichever is larger
static const int64_t kGridStageBytes = std::max<int64_t>((2ll * kTile * 128 + 16ll * kTileElems) * 8, kGridTcStageBytes);

static int chooseBlock(int nrMax, int requested) {
  if (requested == 32 || requested == 64 || requested == 128 || requested == 256) return requested;
  if (nrMax <= 32) return 32;
  if (nrMax <= 64) return 64;
  if (nrMax <= 128) return 128;
  return 256;
}

// The size buckets run concurrently, one persistent launch each. A launch takes every SM it can
// hold as soon as it starts, so with full-GPU grids the buckets launched later only start when
// earlier ones drain their queues, and their slowest instances then end the batch. Instead the
// SMs are apportioned among the buckets in proportion to their estimated work, so that every
// bucket's CTAs are resident from the start and the buckets finish together. Measured on the
// contact batch, the SM time of an instance's iteration grows about linearly with its root size
// nr: about 5 us x nr where a CTA has its SM to itself, about 3 us x nr where several CTAs share
// one (their latency-bound chains overlap). A bucket's work is therefore the sum of its
// instances' nr, times 0.6 for launch shapes with several CTAs per SM (iteration counts are
// alike across buckets). A bucket never gets more SMs than its instances can fill; the rest go
// to the others (largest-remainder apportionment).
static void partitionGrids(cxg_batch* B, int numSM) {
  const size_t G = B->groups.size();
  if (B->gridMode) {  // one cooperative launch over every SM
    for (Group& g : B->groups) g.gridAlone = g.grid;
    return;
  }
  for (Group& g : B->groups) g.gridAlone = std::max(1, std::min(g.count, g.occupancy * numSM));
  if (G <= 1 || (int)G > numSM) {
    for (Group& g : B->groups) g.grid = g.gridAlone;
    return;
  }
  std::vector<int> sms(G, 0), need(G);
  std::vector<bool> capped(G, false);
  auto weight = [&](size_t b) {
    const Group& g = B->groups[b];
    return std::max(g.work, 1.0) * (g.occupancy > 1 ? 0.6 : 1.0);
  };
  for (size_t b = 0; b < G; ++b) {
    const Group& g = B->groups[b];
    need[b] = std::max(1, (g.count + g.occupancy - 1) / g.occupancy);
  }
  int freeSM = numSM;
  for (bool again = true; again;) {
    again = false;
    double w = 0.0;
    for (size_t b = 0; b < G; ++b)
      if (!capped[b]) w += weight(b);
    for (size_t b = 0; b < G && !again; ++b) {
      if (capped[b]) continue;
      const double share = freeSM * weight(b) / w;
      if (share >= need[b]) {  // more SMs than its instances fill: give it what it can use
        sms[b] = need[b];
        capped[b] = true;
        freeSM -= need[b];
        again = true;
      }
    }
  }
  double w = 0.0;
  int open = 0;
  for (size_t b = 0; b < G; ++b)
    if (!capped[b]) {
      w += weight(b);
      ++open;
    }
  if (open > 0) {
    std::vector<std::pair<double, size_t>> frac;
    int used = 0;
    for (size_t b = 0; b < G; ++b) {
      if (capped[b]) continue;
      const double share = std::max(freeSM, open) * weight(b) / w;
      sms[b] = std::max(1, (int)share);
      used += sms[b];
      frac.push_back({share - (double)(int)share, b});
    }
    std::sort(frac.begin(), frac.end(), [](const std::pair<double, size_t>& a, const std::pair<double, size_t>& c) {
      return a.first > c.first;
    });
    for (size_t k = 0; used < freeSM && k < frac.size(); ++k, ++used) sms[frac[k].second] += 1;
  }
  for (size_t b = 0; b < G; ++b) {
    Group& g = B->groups[b];
    g.grid = std::max(1, std::min(g.count, sms[b] * g.occupancy));
  }
}

static int buildGroups(cxg_batch* B) {
  const int N = B->count;
  const bool fp32 = B->st.precision == CXG_PRECISION_MIXED;
  const bool gridMode = B->gridMode;
  int dev = 0;
  CX_CUDA(cudaGetDevice(&dev));
  B->device = dev;
  int smemOptin = 0, numSM = 0;
  CX_CUDA(cudaDeviceGetAttribute(&smemOptin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  CX_CUDA(cudaDeviceGetAttribute(&numSM, cudaDevAttrMultiProcessorCount, dev));
  const size_t fixedSmem = 1024;  // static __shared__ (Ctx, queue slot) and alignment slack
  // order: by bucket (descending nr), then by cost descending
  std::vector<int> idx((size_t)N);
  std::iota(idx.begin(), idx.end(), 0);
  const std::vector<int> edges =
      B->edges.empty() ? std::vector<int>(std::begin(kBucketEdges), std::end(kBucketEdges)) : B->edges;
  auto bucketOf = [&](int nr) {
    int b = 0;
    for (int e : edges) {
      if (nr <= e) return b;
      ++b;
    }
    return b;
  };
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
    const int ba = bucketOf(B->pools.desc[(size_t)a].nr), bb = bucketOf(B->pools.desc[(size_t)b].nr);
    if (ba != bb) return ba > bb;
    return B->pools.desc[(size_t)a].cost > B->pools.desc[(size_t)b].cost;
  });
  B->order = idx;
  B->groups.clear();
  int64_t scratchTotal = 0;
  for (int s = 0; s < N;) {
    int e = s;
    const int bk = bucketOf(B->pools.desc[(size_t)idx[(size_t)s]].nr);
    while (e < N && bucketOf(B->pools.desc[(size_t)idx[(size_t)e]].nr) == bk) ++e;
    Group g;
    g.begin = s;
    g.count = e - s;
    g.fp32 = fp32;
    SmemLayout& L = g.lay;
    L.nMax = L.mMax = L.nrMax = L.nsocMax = 0;
    for (int t = s; t < e; ++t) {
      const InstanceDesc& D = B->pools.desc[(size_t)idx[(size_t)t]];
      L.nMax = std::max(L.nMax, D.n);
      L.mMax = std::max(L.mMax, D.m);
      L.nrMax = std::max(L.nrMax, D.nr);
      L.nsocMax = std::max(L.nsocMax, D.nsoc);
      g.work += (double)D.nr;  // scaled by the launch shape's sharing in partitionGrids
    }
    const int64_t redBytes = (128 + 32) * 8;
    const int64_t vecBytes = vecDoubles(L.nMax, L.mMax, L.nrMax, L.nsocMax) * 8;
    const int64_t root32Bytes = rootSize(L.nrMax) * 4, root64Bytes = rootSize(L.nrMax) * 8;
    const int64_t budget = (int64_t)smemOptin - (int64_t)fixedSmem;
    L.redOff = 0;
    L.vecOff = redBytes;
    // whole-GPU form: everything the other CTAs read (vectors, root, solve vector) in scratch
    L.vecInSmem = (!gridMode && redBytes + vecBytes <= budget) ? 1 : 0;
    int64_t used = redBytes + (L.vecInSmem ? vecBytes : 0);
    used = (used + 15) & ~int64_t(15);
    L.rootOff = used;
    // FP64 root (FP64 precision, or the mixed-precision fallback) in shared memory when it fits;
    // the FP32 root then shares that region.
    L.rootInSmem = 0;
    L.root64InSmem = 0;
    if (!gridMode && used + root64Bytes <= budget) {
      L.rootInSmem = 1;
      L.root64InSmem = 1;
      used += root64Bytes;
    } else if (!gridMode && fp32 && used + root32Bytes <= budget) {
      L.rootInSmem = 1;
      used += root32Bytes;
    }
    if (gridMode) {
      // tile staging area of the whole-GPU trailing update, where the root would otherwise go
      used += kGridStageBytes;
    }
    L.total = used;
    g.smem = (size_t)used;
    g.block = gridMode ? 256 : chooseBlock(L.nrMax, B->st.threads_per_instance);
    // per-instance scratch layout (relative to the CTA base); the FP64 root is needed when the
    // root is not in shared memory (FP64 precision) or for the mixed-precision fallback.
    const bool needRoot64 = !L.root64InSmem;
    int64_t stride = 0;
    for (int t = s; t < e; ++t) {
      InstanceDesc& D = B->pools.desc[(size_t)idx[(size_t)t]];
      int64_t o = 0;
      D.sPv = o; o += r2((int64_t)D.nnzPu + D.nnzPs);
      D.sAv = o; o += r2(D.nnzA);
      D.sAd = o; o += r2(D.nAd);
      D.sT = o; o += r2(D.nAd);
      D.sQ = o; o += r2(D.n);
      D.sB = o; o += r2(D.m);
      D.sRoot64 = o; o += needRoot64 ? r2(rootSize(D.nr)) : 0;
      D.sVec = o; o += L.vecInSmem ? 0 : vecDoubles(L.nMax, L.mMax, L.nrMax, L.nsocMax);
      D.sVecG = o; o += vecGlobalDoubles(L.mMax);
      D.sKry = o; o += gridMode ? krylovDoubles(L.nMax, L.mMax) : 0;
      o = r2(o);  // 16-byte aligned: the slices are read by bulk copies
      D.sSlice = o; o += (gridMode && fp32) ? r2((dfSliceBytes(D.nr) + 7) / 8) : 0;
      D.scratchDoubles = o;
      stride = std::max(stride, o);
    }
    g.stride = std::max<int64_t>(r2(stride), 2);
    // persistent grid: resident CTAs for this configuration, capped by the group size
    int occ = 0;
    if (gridMode) {
      // cooperative launch: every CTA resident; only CTA 0 holds an instance (and scratch)
      CX_CUDA(ipmGridOccupancy(&occ, g.smem, fp32));
      if (occ * numSM < 2) return setErr(CXG_E_UNSUPPORTED, "the whole-GPU root needs two resident CTAs");
      g.grid = occ * numSM;
      g.occupancy = 1;
      g.scratchOff = scratchTotal;
      scratchTotal += g.stride;
    } else {
      const cudaError_t oe = ipmOccupancy(&occ, g.block, g.smem, fp32);
      if (oe != cudaSuccess || occ < 1) occ = 1;
      g.grid = std::max(1, std::min(g.count, occ * numSM));
      g.gridAlone = g.grid;
      g.occupancy = occ;
      g.scratchOff = scratchTotal;
      scratchTotal += g.stride * g.grid;
    }
    g.counterIdx = (int)B->groups.size();
    B->groups.push_back(g);
    s = e;
  }
  partitionGrids(B, numSM);
  scratchTotal = 0;
  for (Group& g : B->groups) {
    g.scratchOff = scratchTotal;
    // the whole-GPU form: only CTA 0 holds the instance, so one scratch region
    scratchTotal += gridMode ? g.stride : g.stride * g.grid;
  }
  // scratch
  if (B->dScratch) cudaFree(B->dScratch);
  B->dScratch = nullptr;
  int rc = devAlloc(&B->dScratch, (size_t)std::max<int64_t>(scratchTotal, 2));
  if (rc) return rc;
  B->scratchCapacity = std::max<int64_t>(scratchTotal, 2);
  return CXG_OK;
}

// After buildGroups on a batch already on the device: the per-bucket queue counters, the
// instance descriptors (their scratch offsets) and the queue order; the captured graph is stale.
static int refreshGroupsOnDevice(cxg_batch* B) {
  const size_t N = (size_t)B->count;
  if (B->dCounters) cudaFree(B->dCounters);
  B->dCounters = nullptr;
  if (int rc = devAlloc(&B->dCounters, B->groups.size() + 1)) return rc;
  CX_CUDA(cudaMemcpy(B->dDesc, B->pools.desc.data(), N * sizeof(InstanceDesc), cudaMemcpyHostToDevice));
  CX_CUDA(cudaMemcpy(B->dOrder, B->order.data(), N * sizeof(int), cudaMemcpyHostToDevice));
  B->graphValid = false;
  return CXG_OK;
}

static int uploadPlan(cxg_batch* B) {
  const size_t N = (size_t)B->count;
  int rc;
  if ((rc = devAlloc(&B->dDesc, N))) return rc;
  if ((rc = devAlloc(&B->dIpool, B->pools.ipool.size()))) return rc;
  if ((rc = devAlloc(&B->dDpool, B->pools.dpool.size()))) return rc;
  B->ipoolCap = std::max<size_t>(B->pools.ipool.size(), 1);
  B->dpoolCap = std::max<size_t>(B->pools.dpool.size(), 1);
  if ((rc = devAlloc(&B->dPx, (size_t)B->pools.totPx))) return rc;
  if ((rc = devAlloc(&B->dq, (size_t)B->pools.totQ))) return rc;
  if ((rc = devAlloc(&B->dAx, (size_t)B->pools.totAx))) return rc;
  if ((rc = devAlloc(&B->db, (size_t)B->pools.totB))) return rc;
  if ((rc = devAlloc(&B->dx, (size_t)B->pools.totQ))) return rc;
  if ((rc = devAlloc(&B->ds, (size_t)B->pools.totB))) return rc;
  if ((rc = devAlloc(&B->dz, (size_t)B->pools.totB))) return rc;
  if ((rc = devAlloc(&B->dRes, N))) return rc;
  if ((rc = devAlloc(&B->dWx, (size_t)B->pools.totQ))) return rc;
  if ((rc = devAlloc(&B->dWs, (size_t)B->pools.totB))) return rc;
  if ((rc = devAlloc(&B->dWz, (size_t)B->pools.totB))) return rc;
  if ((rc = devAlloc(&B->dHaveWarm, N))) return rc;
  if ((rc = devAlloc(&B->dCounters, B->groups.size() + 1))) return rc;
  if ((rc = devAlloc(&B->dOrder, N))) return rc;
  if (B->gridMode && (rc = devAlloc(reinterpret_cast<unsigned char**>(&B->dGridCtl), gridCtlBytes()))) return rc;
  if (B->st.differentiable) {
    if ((rc = devAlloc(&B->dBwd, (size_t)B->bwdTotal))) return rc;
    if ((rc = devAlloc(&B->dGx, (size_t)B->pools.totQ))) return rc;
    if ((rc = devAlloc(&B->dGq, (size_t)B->pools.totQ))) return rc;
    if ((rc = devAlloc(&B->dGb, (size_t)B->pools.totB))) return rc;
    if ((rc = devAlloc(&B->dGP, (size_t)B->pools.totPx))) return rc;
    if ((rc = devAlloc(&B->dGA, (size_t)B->pools.totAx))) return rc;
  }
  CX_CUDA(cudaMemcpy(B->dDesc, B->pools.desc.data(), N * sizeof(InstanceDesc), cudaMemcpyHostToDevice));
  if (!B->pools.ipool.empty())
    CX_CUDA(cudaMemcpy(B->dIpool, B->pools.ipool.data(), B->pools.ipool.size() * sizeof(int), cudaMemcpyHostToDevice));
  if (!B->pools.dpool.empty())
    CX_CUDA(cudaMemcpy(B->dDpool, B->pools.dpool.data(), B->pools.dpool.size() * sizeof(double), cudaMemcpyHostToDevice));
  CX_CUDA(cudaMemcpy(B->dOrder, B->order.data(), N * sizeof(int), cudaMemcpyHostToDevice));
  CX_CUDA(cudaMemset(B->dHaveWarm, 0, N));
  return CXG_OK;
}

// Plans problems[j] into dst[slots[j]], j < k, each into its own pool (offsets from 0), on
// worker threads over contiguous chunks. Throws LimitError / std::exception as planInstance does.
static void planInstances(const cxg_problem* problems, const int* slots, int k, const cxg_settings& st,
                          std::vector<Pools>& dst) {
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  const int nth = std::max(1, std::min({hw, 32, k / 16}));
  std::vector<std::string> fail((size_t)nth);
  std::vector<char> failLimit((size_t)nth, 0);
  auto work = [&](int t) {
    const int lo = (int)((int64_t)k * t / nth), hi = (int)((int64_t)k * (t + 1) / nth);
    try {
      for (int j = lo; j < hi; ++j) {
        Pools one;
        planInstance(problems[j], st, one);
        dst[(size_t)slots[j]] = std::move(one);
      }
    } catch (const LimitError& ex) {
      fail[(size_t)t] = ex.what();
      failLimit[(size_t)t] = 1;
    } catch (const std::exception& ex) {
      fail[(size_t)t] = ex.what();
    }
  };
  if (nth == 1) {
    work(0);
  } else {
    std::vector<std::thread> pool;
    pool.reserve((size_t)nth);
    for (int t = 0; t < nth; ++t) pool.emplace_back(work, t);
    for (std::thread& th : pool) th.join();
  }
  for (int t = 0; t < nth; ++t)
    if (!fail[(size_t)t].empty()) {
      if (failLimit[(size_t)t]) throw LimitError(fail[(size_t)t]);
      throw std::runtime_error(fail[(size_t)t]);
    }
}

// The checks of cxg_batch_create on instance i of a batch of `count` (CXG_OK, or the error code
// with the message set).
static int checkBatchProblem(const cxg_problem& pr, int i, int count, const cxg_settings& st);

static std::string checkFinite(const double* v, int64_t n, const char* name) {
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(v[i])) return std::string(name) + " contains a non-finite value";
  return "";
}

static int checkBatchProblem(const cxg_problem& pr, int i, int count, const cxg_settings& st) {
  std::string e = validateProblem(pr);
  if (!e.empty()) return setErr(CXG_E_INVALID, "instance " + std::to_string(i) + ": " + e);
  e = checkPlanCounts(pr);
  if (!e.empty()) return setErr(CXG_E_UNSUPPORTED, "instance " + std::to_string(i) + ": " + e);
  e = checkFinite(pr.Px, pr.Pp[pr.n], "P");
  if (e.empty()) e = checkFinite(pr.Ax, pr.Ap[pr.n], "A");
  if (e.empty()) e = checkFinite(pr.q, pr.n, "q");
  if (e.empty()) e = checkFinite(pr.b, pr.m, "b");
  if (!e.empty()) return setErr(CXG_E_INVALID, "instance " + std::to_string(i) + ": " + e);
  const int nr = pr.n + pr.zero_dim;
  if (nr > kCtaMaxRoot && !(count == 1 && st.whole_gpu_root >= 0 && nr <= kGridMaxRoot))
    return setErr(CXG_E_UNSUPPORTED,
                  "instance " + std::to_string(i) + ": n + zero_dim = " + std::to_string(nr) +
                      " exceeds the one-CTA root (4096 rows); a single instance (count 1, whole_gpu_root >= 0) "
                      "takes the whole-GPU root up to " + std::to_string(kGridMaxRoot) + " rows");
  return CXG_OK;
}

extern "C" int cxg_batch_create(cxg_batch** out, int count, const cxg_problem* problems,
                                const cxg_settings* settings) {
  if (!out) return setErr(CXG_E_INVALID, "null output handle");
  *out = nullptr;
  if (count < 1 || !problems) return setErr(CXG_E_INVALID, "count must be >= 1");
  const auto t0 = std::chrono::steady_clock::now();
  cxg_settings st;
  if (settings) st = *settings;
  else {
    cxg_default_settings(&st);
    st.precision = CXG_PRECISION_MIXED;
  }
  for (int i = 0; i < count; ++i)
    if (int rc = checkBatchProblem(problems[i], i, count, st)) return rc;
  // One instance whose root one CTA cannot hold, or when asked: spread the root over every SM.
  // (cxg_solver_setup asks for it from kGridAutoRoot rows on.)
  const int nr0 = problems[0].n + problems[0].zero_dim;
  const bool gridMode = count == 1 && (st.whole_gpu_root == 1 || nr0 > kCtaMaxRoot);
  // the adjoint keeps an FP64 copy of the final factor and solves with it on one CTA: offered up
  // to 8192 root rows
  const bool bwdDropped = gridMode && nr0 > kGridMaxAdjointRoot && st.differentiable;
  if (bwdDropped) st.differentiable = 0;
  cxg_batch* B = new (std::nothrow) cxg_batch();
  if (!B) return setErr(CXG_E_NOMEM, "host allocation failed");
  B->count = count;
  B->st = st;
  B->kktSt = st;
  B->gridMode = gridMode;
  B->bwdDropped = bwdDropped;
  try {
    // Host planning, the set-up cost when contact patterns change: contiguous chunks of instances
    // are planned on worker threads into their own pools, then appended in instance order.
    B->inst.resize((size_t)count);
    std::vector<int> all((size_t)count);
    std::iota(all.begin(), all.end(), 0);
    planInstances(problems, all.data(), count, st, B->inst);
    for (const Pools& pp : B->inst) appendPools(B->pools, pp);
    for (int i = 0; i < count; ++i) {
      const cxg_problem& pr = problems[i];
      B->Pp.emplace_back(pr.Pp, pr.Pp + pr.n + 1);
      B->Pi.emplace_back(pr.Pi, pr.Pi + pr.Pp[pr.n]);
      B->Ap.emplace_back(pr.Ap, pr.Ap + pr.n + 1);
      B->Ai.emplace_back(pr.Ai, pr.Ai + pr.Ap[pr.n]);
    }
  } catch (const LimitError& ex) {
    delete B;
    return setErr(CXG_E_UNSUPPORTED, std::string("planning refused: ") + ex.what());
  } catch (const std::exception& ex) {
    delete B;
    return setErr(CXG_E_NOMEM, std::string("planning failed: ") + ex.what());
  }
  if (st.differentiable) {
    int64_t off = 0;
    for (InstanceDesc& D : B->pools.desc) {
      D.bwdOff = off;
      off += bwdLayout(D.nr, D.n, D.m, D.nsoc).total;
    }
    B->bwdTotal = off;
  }
  int rc = CXG_OK;
  if (cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete B;
    return setErr(CXG_E_CUDA, "cudaStreamCreate failed (no CUDA device?)");
  }
  if ((rc = buildGroups(B)) || (rc = uploadPlan(B))) {
    delete B;
    return rc;
  }
  // initial values
  std::vector<double> hv;
  auto upload = [&](double* dst, int64_t total, int which) -> int {
    hv.assign((size_t)std::max<int64_t>(total, 1), 0.0);
    for (int i = 0; i < count; ++i) {
      const cxg_problem& pr = problems[i];
      const InstanceDesc& D = B->pools.desc[(size_t)i];
      if (which == 0) std::copy(pr.Px, pr.Px + D.nnzPu, hv.begin() + D.vPx);
      if (which == 1) std::copy(pr.q, pr.q + D.n, hv.begin() + D.vQ);
      if (which == 2) std::copy(pr.Ax, pr.Ax + D.nnzA, hv.begin() + D.vAx);
      if (which == 3) std::copy(pr.b, pr.b + D.m, hv.begin() + D.vB);
    }
    if (total > 0) CX_CUDA(cudaMemcpy(dst, hv.data(), (size_t)total * sizeof(double), cudaMemcpyHostToDevice));
    return CXG_OK;
  };
  if ((rc = upload(B->dPx, B->pools.totPx, 0)) || (rc = upload(B->dq, B->pools.totQ, 1)) ||
      (rc = upload(B->dAx, B->pools.totAx, 2)) || (rc = upload(B->db, B->pools.totB, 3))) {
    delete B;
    return rc;
  }
  B->hRes.resize((size_t)count);
  B->setupTime = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  *out = B;
  return CXG_OK;
}

// ------------------------------------------------------------------------------------------
// replacing instances (new patterns) without a new batch
// ------------------------------------------------------------------------------------------
// Per-instance arrays of a batch, in the concatenated layouts: values (P, q, A, b), solutions and
// warm starts. moveKernel copies each kept instance's segments from the old layout to the new one
// (one CTA per instance).
struct MoveArgs {
  static constexpr int kArrays = 10;
  const double* src[kArrays];
  double* dst[kArrays];
  int kind[kArrays];          // 0: P values, 1: n-vector, 2: A values, 3: m-vector
  const int64_t* oldOff;      // count x 4: vPx, vQ, vAx, vB of the old layout
  const int64_t* newOff;      // count x 4, new layout
  const int64_t* len;         // count x 4: nnzP, n, nnzA, m
  const unsigned char* keep;  // count
};

__global__ void __launch_bounds__(256) moveKernel(MoveArgs a, int count) {
  const int i = blockIdx.x;
  if (i >= count || !a.keep[i]) return;
  for (int k = 0; k < MoveArgs::kArrays; ++k) {
    if (!a.src[k]) continue;
    const int kd = a.kind[k];
    const int64_t so = a.oldOff[4 * i + kd], dof = a.newOff[4 * i + kd], ln = a.len[4 * i + kd];
    for (int64_t t = threadIdx.x; t < ln; t += blockDim.x) a.dst[k][dof + t] = a.src[k][so + t];
  }
}

extern "C" int cxg_batch_replace(cxg_batch* B, int k, const int* indices, const cxg_problem* problems) {
  if (!B) return setErr(CXG_E_INVALID, "null batch");
  if (k < 0 || (k > 0 && (!indices || !problems))) return setErr(CXG_E_INVALID, "null indices or problems");
  if (k == 0) return CXG_OK;
  if (B->gridMode) return setErr(CXG_E_UNSUPPORTED, "a whole-GPU single instance is set up anew with cxg_solver_setup");
  std::vector<char> seen((size_t)B->count, 0);
  for (int j = 0; j < k; ++j) {
    const int i = indices[j];
    if (i < 0 || i >= B->count) return setErr(CXG_E_INVALID, "instance index out of range");
    if (seen[(size_t)i]) return setErr(CXG_E_INVALID, "instance index repeated");
    seen[(size_t)i] = 1;
    if (int rc = checkBatchProblem(problems[j], i, B->count, B->kktSt)) return rc;
  }
  const auto t0 = std::chrono::steady_clock::now();
  CX_CUDA(cudaSetDevice(B->device));
  CX_CUDA(cudaStreamSynchronize(B->stream));
  // (1) host plans of the new instances, then the concatenated pools in instance order
  std::vector<Pools> fresh((size_t)B->count);
  try {
    planInstances(problems, indices, k, B->kktSt, fresh);
  } catch (const LimitError& ex) {
    return setErr(CXG_E_UNSUPPORTED, std::string("planning refused: ") + ex.what());
  } catch (const std::exception& ex) {
    return setErr(CXG_E_NOMEM, std::string("planning failed: ") + ex.what());
  }
  const std::vector<InstanceDesc> oldDesc = B->pools.desc;
  // The new plans go after the pool's end (the replaced instances' old blocks stay as unused
  // space, so only the tail is uploaded); when unused space would exceed the live plans, the
  // pool is rebuilt from the per-instance plans.
  const size_t oldI = B->pools.ipool.size(), oldD = B->pools.dpool.size();
  size_t liveI = 0, newI = 0;
  for (int j = 0; j < k; ++j) newI += fresh[(size_t)indices[j]].ipool.size() + 1;
  for (const Pools& pp : B->inst) liveI += pp.ipool.size() + 1;
  for (int j = 0; j < k; ++j) liveI -= B->inst[(size_t)indices[j]].ipool.size() + 1;
  liveI += newI;
  const bool compact = oldI + newI > 2 * liveI + (size_t(1) << 20);
  for (int j = 0; j < k; ++j) {
    const int i = indices[j];
    B->inst[(size_t)i] = std::move(fresh[(size_t)i]);
    const cxg_problem& pr = problems[j];
    B->Pp[(size_t)i].assign(pr.Pp, pr.Pp + pr.n + 1);
    B->Pi[(size_t)i].assign(pr.Pi, pr.Pi + pr.Pp[pr.n]);
    B->Ap[(size_t)i].assign(pr.Ap, pr.Ap + pr.n + 1);
    B->Ai[(size_t)i].assign(pr.Ai, pr.Ai + pr.Ap[pr.n]);
    if (!compact) {
      appendPools(B->pools, B->inst[(size_t)i]);
      B->pools.desc[(size_t)i] = B->pools.desc.back();
      B->pools.desc.pop_back();
    }
  }
  if (compact) {
    Pools np;
    for (const Pools& pp : B->inst) appendPools(np, pp);
    B->pools = std::move(np);
  } else {
    // the value arrays stay in instance order: offsets from the instances' sizes
    int64_t oPx = 0, oQ = 0, oAx = 0, oB = 0;
    for (InstanceDesc& D : B->pools.desc) {
      D.vPx = oPx; D.vQ = oQ; D.vAx = oAx; D.vB = oB;
      D.vX = D.vQ; D.vS = D.vB; D.vZ = D.vB;
      oPx += D.nnzPu; oQ += D.n; oAx += D.nnzA; oB += D.m;
    }
    B->pools.totPx = oPx; B->pools.totQ = oQ; B->pools.totAx = oAx; B->pools.totB = oB;
  }
  if (B->st.differentiable) {
    int64_t off = 0;
    for (InstanceDesc& D : B->pools.desc) {
      D.bwdOff = off;
      off += bwdLayout(D.nr, D.n, D.m, D.nsoc).total;
    }
    B->bwdTotal = off;
  }
  // (2) the per-instance device arrays in the new layout: kept instances' values, solutions and
  //     warm starts moved on the device, the new instances' values uploaded, their warm starts off
  const size_t N = (size_t)B->count;
  std::vector<int64_t> oldOff(4 * N), newOff(4 * N), len(4 * N);
  std::vector<unsigned char> keep(N, 1);
  for (int j = 0; j < k; ++j) keep[(size_t)indices[j]] = 0;
  for (size_t i = 0; i < N; ++i) {
    const InstanceDesc &O = oldDesc[i], &D = B->pools.desc[i];
    oldOff[4 * i] = O.vPx; oldOff[4 * i + 1] = O.vQ; oldOff[4 * i + 2] = O.vAx; oldOff[4 * i + 3] = O.vB;
    newOff[4 * i] = D.vPx; newOff[4 * i + 1] = D.vQ; newOff[4 * i + 2] = D.vAx; newOff[4 * i + 3] = D.vB;
    len[4 * i] = D.nnzPu; len[4 * i + 1] = D.n; len[4 * i + 2] = D.nnzA; len[4 * i + 3] = D.m;
  }
  double* na[MoveArgs::kArrays] = {};
  double** olds[MoveArgs::kArrays] = {&B->dPx, &B->dq, &B->dAx, &B->db, &B->dx, &B->ds, &B->dz, &B->dWx, &B->dWs, &B->dWz};
  const int kinds[MoveArgs::kArrays] = {0, 1, 2, 3, 1, 3, 3, 1, 3, 3};
  const int64_t totals[4] = {B->pools.totPx, B->pools.totQ, B->pools.totAx, B->pools.totB};
  int64_t* dOld = nullptr;
  int64_t* dNew = nullptr;
  int64_t* dLen = nullptr;
  unsigned char* dKeep = nullptr;
  int rc = CXG_OK;
  auto cleanup = [&]() {
    for (double* p : na) if (p) cudaFree(p);
    if (dOld) cudaFree(dOld);
    if (dNew) cudaFree(dNew);
    if (dLen) cudaFree(dLen);
    if (dKeep) cudaFree(dKeep);
  };
  for (int a = 0; a < MoveArgs::kArrays && !rc; ++a) rc = devAlloc(&na[a], (size_t)std::max<int64_t>(totals[kinds[a]], 1));
  if (!rc) rc = devAlloc(&dOld, 4 * N);
  if (!rc) rc = devAlloc(&dNew, 4 * N);
  if (!rc) rc = devAlloc(&dLen, 4 * N);
  if (!rc) rc = devAlloc(&dKeep, N);
  if (rc) { cleanup(); return rc; }
  cudaError_t ce = cudaMemcpy(dOld, oldOff.data(), 4 * N * sizeof(int64_t), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(dNew, newOff.data(), 4 * N * sizeof(int64_t), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(dLen, len.data(), 4 * N * sizeof(int64_t), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(dKeep, keep.data(), N, cudaMemcpyHostToDevice);
  // the new instances' values at their new offsets, their solutions and warm starts zero
  for (int a = 0; a < MoveArgs::kArrays && ce == cudaSuccess; ++a)
    if (a >= 4) ce = cudaMemset(na[a], 0, (size_t)std::max<int64_t>(totals[kinds[a]], 1) * sizeof(double));
  for (int j = 0; j < k && ce == cudaSuccess; ++j) {
    const cxg_problem& pr = problems[j];
    const InstanceDesc& D = B->pools.desc[(size_t)indices[j]];
    if (D.nnzPu) ce = cudaMemcpy(na[0] + D.vPx, pr.Px, (size_t)D.nnzPu * sizeof(double), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess && D.n) ce = cudaMemcpy(na[1] + D.vQ, pr.q, (size_t)D.n * sizeof(double), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess && D.nnzA) ce = cudaMemcpy(na[2] + D.vAx, pr.Ax, (size_t)D.nnzA * sizeof(double), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess && D.m) ce = cudaMemcpy(na[3] + D.vB, pr.b, (size_t)D.m * sizeof(double), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemset(B->dHaveWarm + indices[j], 0, 1);
  }
  if (ce == cudaSuccess) {
    MoveArgs ma{};
    for (int a = 0; a < MoveArgs::kArrays; ++a) {
      ma.src[a] = *olds[a];
      ma.dst[a] = na[a];
      ma.kind[a] = kinds[a];
    }
    ma.oldOff = dOld;
    ma.newOff = dNew;
    ma.len = dLen;
    ma.keep = dKeep;
    moveKernel<<<B->count, 256>>>(ma, B->count);
    ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
  }
  if (ce != cudaSuccess) {
    cleanup();
    return setErr(CXG_E_CUDA, std::string("replace: ") + cudaGetErrorString(ce));
  }
  for (int a = 0; a < MoveArgs::kArrays; ++a) {
    cudaFree(*olds[a]);
    *olds[a] = na[a];
    na[a] = nullptr;
  }
  cleanup();
  // (3) the plan arrays, the size buckets (grids, scratch, counters) and the saved adjoint states
  if ((rc = buildGroups(B))) return rc;
  if ((rc = refreshGroupsOnDevice(B))) return rc;
  // pool arrays: the new tail only, unless they were rebuilt or outgrew the capacity
  auto syncPool = [&](auto*& dptr, size_t& cap, const auto& host, size_t oldSize) -> int {
    using E = typename std::decay<decltype(host[0])>::type;
    const size_t nsz = host.size();
    size_t from = compact ? 0 : oldSize;
    if (nsz > cap) {
      const size_t ncap = nsz + nsz / 2;
      E* np_ = nullptr;
      if (int r = devAlloc(&np_, ncap)) return r;
      if (!compact && oldSize) {
        const cudaError_t e2 = cudaMemcpy(np_, dptr, oldSize * sizeof(E), cudaMemcpyDeviceToDevice);
        if (e2 != cudaSuccess) { cudaFree(np_); return setErr(CXG_E_CUDA, cudaGetErrorString(e2)); }
      }
      cudaFree(dptr);
      dptr = np_;
      cap = ncap;
    }
    if (nsz > from) {
      const cudaError_t e2 = cudaMemcpy(dptr + from, host.data() + from, (nsz - from) * sizeof(E), cudaMemcpyHostToDevice);
      if (e2 != cudaSuccess) return setErr(CXG_E_CUDA, cudaGetErrorString(e2));
    }
    return CXG_OK;
  };
  if ((rc = syncPool(B->dIpool, B->ipoolCap, B->pools.ipool, oldI))) return rc;
  if ((rc = syncPool(B->dDpool, B->dpoolCap, B->pools.dpool, oldD))) return rc;
  if (B->st.differentiable) {
    double* g[6] = {B->dBwd, B->dGx, B->dGq, B->dGb, B->dGP, B->dGA};
    for (double* p : g)
      if (p) cudaFree(p);
    B->dBwd = B->dGx = B->dGq = B->dGb = B->dGP = B->dGA = nullptr;
    if ((rc = devAlloc(&B->dBwd, (size_t)std::max<int64_t>(B->bwdTotal, 1))) ||
        (rc = devAlloc(&B->dGx, (size_t)std::max<int64_t>(B->pools.totQ, 1))) ||
        (rc = devAlloc(&B->dGq, (size_t)std::max<int64_t>(B->pools.totQ, 1))) ||
        (rc = devAlloc(&B->dGb, (size_t)std::max<int64_t>(B->pools.totB, 1))) ||
        (rc = devAlloc(&B->dGP, (size_t)std::max<int64_t>(B->pools.totPx, 1))) ||
        (rc = devAlloc(&B->dGA, (size_t)std::max<int64_t>(B->pools.totAx, 1))))
      return rc;
    B->bwdStale = true;
  }
  B->graphValid = false;
  B->setupTime = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return CXG_OK;
}

extern "C" void cxg_batch_destroy(cxg_batch* b) { delete b; }
extern "C" int cxg_batch_count(const cxg_batch* b) { return b ? b->count : 0; }

extern "C" int cxg_batch_sizes(const cxg_batch* b, int64_t* nnzP, int64_t* n, int64_t* nnzA, int64_t* m) {
  if (!b) return setErr(CXG_E_INVALID, "null batch");
  if (nnzP) *nnzP = b->pools.totPx;
  if (n) *n = b->pools.totQ;
  if (nnzA) *nnzA = b->pools.totAx;
  if (m) *m = b->pools.totB;
  return CXG_OK;
}

extern "C" int cxg_batch_offsets(const cxg_batch* b, int i, int64_t* pOff, int64_t* nOff, int64_t* aOff, int64_t* mOff) {
  if (!b || i < 0 || i >= b->count) return setErr(CXG_E_INVALID, "bad batch or index");
  const InstanceDesc& D = b->pools.desc[(size_t)i];
  if (pOff) *pOff = D.vPx;
  if (nOff) *nOff = D.vQ;
  if (aOff) *aOff = D.vAx;
  if (mOff) *mOff = D.vB;
  return CXG_OK;
}

static int copyValues(cxg_batch* B, const double* Px, const double* q, const double* Ax, const double* b,
                      cudaMemcpyKind kind, cudaStream_t s) {
  if (Px && B->pools.totPx) CX_CUDA(cudaMemcpyAsync(B->dPx, Px, (size_t)B->pools.totPx * 8, kind, s));
  if (q && B->pools.totQ) CX_CUDA(cudaMemcpyAsync(B->dq, q, (size_t)B->pools.totQ * 8, kind, s));
  if (Ax && B->pools.totAx) CX_CUDA(cudaMemcpyAsync(B->dAx, Ax, (size_t)B->pools.totAx * 8, kind, s));
  if (b && B->pools.totB) CX_CUDA(cudaMemcpyAsync(B->db, b, (size_t)B->pools.totB * 8, kind, s));
  return CXG_OK;
}

extern "C" int cxg_batch_update_values(cxg_batch* B, const double* Px, const double* q, const double* Ax, const double* b) {
  if (!B) return setErr(CXG_E_INVALID, "null batch");
  int rc = copyValues(B, Px, q, Ax, b, cudaMemcpyHostToDevice, B->stream);
  if (rc) return rc;
  CX_CUDA(cudaStreamSynchronize(B->stream));
  return CXG_OK;
}

extern "C" int cxg_batch_update_values_device(cxg_batch* B, const double* Px, const double* q, const double* Ax,
                                              const double* b, void* stream) {
  if (!B) return setErr(CXG_E_INVALID, "null batch");
  return copyValues(B, Px, q, Ax, b, cudaMemcpyDeviceToDevice, (cudaStream_t)stream);
}

// Arguments of one bucket's IPM launch (counter and scratch base given by the caller).
static LaunchArgs solveArgs(const cxg_batch* B, const Group& g, const DevSettings& ds, int* counter, double* scratch) {
  LaunchArgs a{};
  a.desc = B->dDesc;
  a.order = B->dOrder + g.begin;
  a.count = g.count;
  a.counter = counter;
  a.ipool = B->dIpool;
  a.dpool = B->dDpool;
  a.Px = B->dPx;
  a.q = B->dq;
  a.Ax = B->dAx;
  a.b = B->db;
  a.x = B->dx;
  a.s = B->ds;
  a.z = B->dz;
  a.results = B->dRes;
  a.warmX = B->dWx;
  a.warmS = B->dWs;
  a.warmZ = B->dWz;
  a.haveWarm = B->dHaveWarm;
  a.bwd = B->dBwd;
  a.trace = ds.record_timings ? B->dTrace : nullptr;
  a.traceRows = B->traceRows;
  a.scratch = scratch;
  a.scratchStride = g.stride;
  a.st = ds;
  a.lay = g.lay;
  return a;
}

// record_timings: the iteration-trace buffer, sized for max_iter rows per instance (allocated
// before any graph capture; a larger max_iter re-allocates it and invalidates the graph).
static int ensureTrace(cxg_batch* B) {
  if (!B->st.record_timings) return CXG_OK;
  const int rows = std::max(1, B->st.max_iter);
  if (B->dTrace && B->traceRows >= rows) return CXG_OK;
  if (B->dTrace) cudaFree(B->dTrace);
  B->dTrace = nullptr;
  B->traceRows = 0;
  B->graphValid = false;
  int rc = devAlloc(&B->dTrace, (size_t)B->count * (size_t)rows * kTraceCols);
  if (rc) return rc;
  CX_CUDA(cudaMemset(B->dTrace, 0, sizeof(double) * (size_t)B->count * (size_t)rows * kTraceCols));
  B->traceRows = rows;
  return CXG_OK;
}

// ------------------------------------------------------------------------------------------
// history-ordered queues: after each solve, every size bucket's queue is re-sorted by the cost
// its instances just had (iterations x nr^3, x4 when the instance held the double-float factor),
// so that in a timestep loop the instances that ran longest start first next time. A bucket's
// makespan is set by its slowest instances; started late, they would end the batch late.
// The order only decides which CTA takes an instance and when: each instance's arithmetic, and
// so every result bit, is the same in any order.
// ------------------------------------------------------------------------------------------
constexpr int kSortMax = 4096;  // buckets with more instances keep their set-up order
constexpr int kMaxGroups = 16;
struct GroupRanges {
  int begin[kMaxGroups], count[kMaxGroups];
};

__global__ void __launch_bounds__(1024) reorderKernel(const InstanceDesc* desc, const DevResult* res, int* order,
                                                      GroupRanges gr) {
  __shared__ double key[kSortMax];
  __shared__ int idx[kSortMax];
  const int n = gr.count[blockIdx.x];
  int* o = order + gr.begin[blockIdx.x];
  if (n < 2 || n > kSortMax) return;
  int N = 1;
  while (N < n) N <<= 1;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    if (i < n) {
      const int inst = o[i];
      const DevResult& r = res[inst];
      const int it = r.iterations > 0 ? r.iterations : 1;
      key[i] = desc[inst].cost * (double)it * (r.fp64_fallbacks > 0 ? 4.0 : 1.0);
      idx[i] = inst;
    } else {
      key[i] = -1.0;  // padding sorts last
      idx[i] = 0x7fffffff;
    }
  }
  __syncthreads();
  // bitonic sort, descending key, ties by ascending instance index (deterministic)
  for (int k = 2; k <= N; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const int p = i ^ j;
        if (p > i) {
          const bool before = key[i] > key[p] || (key[i] == key[p] && idx[i] < idx[p]);  // i ahead of p
          const bool desc_ = (i & k) == 0;
          if (desc_ ? !before : before) {
            const double tk = key[i];
            key[i] = key[p];
            key[p] = tk;
            const int ti = idx[i];
            idx[i] = idx[p];
            idx[p] = ti;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) o[i] = idx[i];
}

static int enqueueReorder(cxg_batch* B, cudaStream_t s) {
  const int G = (int)B->groups.size();
  if (G < 1 || G > kMaxGroups) return CXG_OK;
  GroupRanges gr{};
  for (int gi = 0; gi < G; ++gi) {
    gr.begin[gi] = B->groups[(size_t)gi].begin;
    gr.count[gi] = B->groups[(size_t)gi].count;
  }
  reorderKernel<<<G, 1024, 0, s>>>(B->dDesc, B->dRes, B->dOrder, gr);
  CX_CUDA(cudaGetLastError());
  return CXG_OK;
}

// Enqueues the device-side solve sequence on `s`: queue resets, then one persistent launch per
// size bucket, each on its own stream forked from and joined back into `s`, so the buckets run
// concurrently and the batch waits for its slowest instance once rather than once per bucket;
// then the queues are re-ordered for the next solve (history-ordered queues, above).
static int enqueueSolve(cxg_batch* B, cudaStream_t s) {
  const DevSettings ds = makeDevSettings(B->st, B->kktSt);
  CX_CUDA(cudaMemsetAsync(B->dCounters, 0, sizeof(int) * (B->groups.size() + 1), s));
  const size_t G = B->groups.size();
  // one stream per launch rank, the first the highest priority: the block scheduler dispatches
  // pending CTAs by stream priority, so the placement follows the launch order below even where
  // the graph submits its independent launches in another order
  if (B->groupStreams.size() < G) {
    int least = 0, greatest = 0;
    CX_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    while (B->groupStreams.size() < G) {
      const int rank = (int)B->groupStreams.size();
      const int prio = std::min(least, greatest + rank);
      cudaStream_t gs;
      CX_CUDA(cudaStreamCreateWithPriority(&gs, cudaStreamNonBlocking, prio));
      B->groupStreams.push_back(gs);
    }
  }
  while (B->forkJoin.size() < G + 1) {
    cudaEvent_t e;
    CX_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    B->forkJoin.push_back(e);
  }
  if (B->gridMode) {
    const Group& g = B->groups[0];
    CX_CUDA(cudaMemsetAsync(B->dGridCtl, 0, gridCtlBytes(), s));
    const LaunchArgs a = solveArgs(B, g, ds, B->dCounters, B->dScratch + g.scratchOff);
    CX_CUDA(launchIpmGrid(a, reinterpret_cast<GridCtl*>(B->dGridCtl), g.grid, g.smem, g.fp32, s));
    B->lastLaunches = 1;
    return CXG_OK;
  }
  CX_CUDA(cudaEventRecord(B->forkJoin[0], s));
  // Launch order: by shared memory per CTA, largest first. The grids are apportioned so that all
  // of them can be resident at once (partitionGrids); the block scheduler spreads each launch's
  // CTAs over the SMs with room left, so the largest CTAs must be placed before the small ones
  // scatter over every SM and leave no SM with room for a large one (first fit, decreasing).
  std::vector<size_t> launchOrder(G);
  std::iota(launchOrder.begin(), launchOrder.end(), size_t(0));
  std::stable_sort(launchOrder.begin(), launchOrder.end(),
                   [&](size_t a_, size_t b_) { return B->groups[a_].smem > B->groups[b_].smem; });
  for (size_t rank = 0; rank < G; ++rank) {
    const size_t gi = launchOrder[rank];
    const Group& g = B->groups[gi];
    cudaStream_t gs = (G == 1) ? s : B->groupStreams[rank];
    if (G > 1) CX_CUDA(cudaStreamWaitEvent(gs, B->forkJoin[0], 0));
    const LaunchArgs a = solveArgs(B, g, ds, B->dCounters + g.counterIdx, B->dScratch + g.scratchOff);
    CX_CUDA(launchIpm(a, g.grid, g.block, g.smem, g.fp32, gs));
    if (G > 1) {
      CX_CUDA(cudaEventRecord(B->forkJoin[gi + 1], gs));
      CX_CUDA(cudaStreamWaitEvent(s, B->forkJoin[gi + 1], 0));
    }
  }
  int rc = enqueueReorder(B, s);
  if (rc) return rc;
  B->lastLaunches = (int)G + ((G >= 1 && G <= (size_t)kMaxGroups) ? 1 : 0);  // bucket launches + reorder
  return CXG_OK;
}

// Device-side solve through the captured graph (re-captured when the settings change).
static int runSolve(cxg_batch* B, cudaStream_t s) {
  if (int rc = ensureTrace(B)) return rc;
  B->bwdStale = false;
  // the whole-GPU form is one cooperative launch: enqueued directly, not through a graph
  if (B->gridMode) return enqueueSolve(B, s);
  const DevSettings ds = makeDevSettings(B->st, B->kktSt);
  if (!B->graphValid || !sameDev(ds, B->graphSettings)) {
    if (B->graphExec) { cudaGraphExecDestroy(B->graphExec); B->graphExec = nullptr; }
    if (B->graph) { cudaGraphDestroy(B->graph); B->graph = nullptr; }
    B->graphValid = false;
    CX_CUDA(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueueSolve(B, B->stream);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(B->stream, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (ce != cudaSuccess) return setErr(CXG_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
    B->graph = g;
    CX_CUDA(cudaGraphInstantiate(&B->graphExec, B->graph, cudaGraphInstantiateFlagUseNodePriority));
    B->graphSettings = ds;
    B->graphValid = true;
  }
  CX_CUDA(cudaGraphLaunch(B->graphExec, s));
  const size_t G = B->groups.size();
  B->lastLaunches = (int)G + ((G >= 1 && G <= (size_t)kMaxGroups) ? 1 : 0);
  return CXG_OK;
}

static double g_clockHz = 0.0;

static void resultToInfo(const DevResult& R, cxg_info& I, double setupTime, double solveTime) {
  std::memset(&I, 0, sizeof(I));
  I.status = R.status;
  I.iterations = R.iterations;
  I.objective = R.objective;
  I.primal_residual = R.primal_residual;
  I.dual_residual = R.dual_residual;
  I.duality_gap = R.duality_gap;
  I.mu = R.mu;
  I.setup_time_s = setupTime;
  I.solve_time_s = solveTime;
  I.fp64_fallbacks = R.fp64_fallbacks;
  I.refine_steps = R.refine_steps;
  I.max_relres = R.max_relres;
  I.factor_attempts = R.factor_attempts;
  I.escalations = R.escalations;
  if (g_clockHz > 0.0) {
    I.time_factor_s = (double)R.cycles[1] / g_clockHz;
    I.time_kkt_solve_s = (double)R.cycles[2] / g_clockHz;
    I.time_other_s = (double)R.cycles[3] / g_clockHz;
    I.time_assemble_s = (double)R.cycles[4] / g_clockHz;
    I.time_ldlt_s = (double)R.cycles[5] / g_clockHz;
    I.time_dense_solve_s = (double)R.cycles[6] / g_clockHz;
    I.time_residual_s = (double)R.cycles[7] / g_clockHz;
  }
}

static int fetchInfo(cxg_batch* B, cxg_info* info, double solveTime) {
  if (!info) return CXG_OK;
  if (g_clockHz == 0.0) {
    int khz = 0;
    if (cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, B->device) == cudaSuccess && khz > 0) g_clockHz = khz * 1e3;
  }
  CX_CUDA(cudaMemcpy(B->hRes.data(), B->dRes, sizeof(DevResult) * (size_t)B->count, cudaMemcpyDeviceToHost));
  for (int i = 0; i < B->count; ++i) resultToInfo(B->hRes[(size_t)i], info[i], B->setupTime, solveTime);
  if (B->st.record_timings && B->count > 0) {
    long long t0 = B->hRes[0].wall_ns[0];
    for (int i = 1; i < B->count; ++i) t0 = std::min(t0, B->hRes[(size_t)i].wall_ns[0]);
    for (int i = 0; i < B->count; ++i) {
      info[i].time_start_s = 1e-9 * (double)(B->hRes[(size_t)i].wall_ns[0] - t0);
      info[i].time_end_s = 1e-9 * (double)(B->hRes[(size_t)i].wall_ns[1] - t0);
    }
  }
  return CXG_OK;
}

extern "C" int cxg_batch_solve(cxg_batch* B, double* x, double* s, double* z, cxg_info* info) {
  if (!B) return setErr(CXG_E_INVALID, "null batch");
  const auto t0 = std::chrono::steady_clock::now();
  int rc = runSolve(B, B->stream);
  if (rc) return rc;
  if (x && B->pools.totQ) CX_CUDA(cudaMemcpyAsync(x, B->dx, (size_t)B->pools.totQ * 8, cudaMemcpyDeviceToHost, B->stream));
  if (s && B->pools.totB) CX_CUDA(cudaMemcpyAsync(s, B->ds, (size_t)B->pools.totB * 8, cudaMemcpyDeviceToHost, B->stream));
  if (z && B->pools.totB) CX_CUDA(cudaMemcpyAsync(z, B->dz, (size_t)B->pools.totB * 8, cudaMemcpyDeviceToHost, B->stream));
  CX_CUDA(cudaStreamSynchronize(B->stream));
  const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return fetchInfo(B, info, dt);
}

extern "C" int cxg_batch_solve_device(cxg_batch* B, double* x, double* s, double* z, cxg_info* info, void* stream) {
  if (!B) return setErr(CXG_E_INVALID, "null batch");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = runSolve(B, st);
  if (rc) return rc;
  if (x && B->pools.totQ) CX_CUDA(cudaMemcpyAsync(x, B->dx, (size_t)B->pools.totQ * 8, cudaMemcpyDeviceToDevice, st));
  if (s && B->pools.totB) CX_CUDA(cudaMemcpyAsync(s, B->ds, (size_t)B->pools.totB * 8, cudaMemcpyDeviceToDevice, st));
  if (z && B->pools.totB) CX_CUDA(cudaMemcpyAsync(z, B->dz, (size_t)B->pools.totB * 8, cudaMemcpyDeviceToDevice, st));
  if (info) {
    CX_CUDA(cudaStreamSynchronize(st));
    return fetchInfo(B, info, 0.0);
  }
  return CXG_OK;
}

extern "C" int cxg_batch_last_launches(const cxg_batch* B) { return B ? B->lastLaunches : 0; }

extern "C" int cxg_batch_footprint(const cxg_batch* B, int64_t* plan, int64_t* values, int64_t* scratch) {
  if (!B) return setErr(CXG_E_INVALID, "null batch");
  if (plan)
    *plan = (int64_t)(B->pools.ipool.size() * sizeof(int) + B->pools.dpool.size() * sizeof(double) +
                      B->pools.desc.size() * sizeof(InstanceDesc) + B->order.size() * sizeof(int));
  if (values)
    *values = 8 * (B->pools.totPx + B->pools.totAx + 2 * B->pools.totQ + 3 * B->pools.totB) +
              (int64_t)(B->count * sizeof(DevResult));
  if (scratch) {
    int64_t t = 0;
    for (const Group& g : B->groups) t += g.stride * g.grid * 8;
    *scratch = t;
  }
  return CXG_OK;
}

extern "C" int cxg_batch_describe(const cxg_batch* B, char* buf, int buflen) {
  if (!B || !buf || buflen <= 0) return setErr(CXG_E_INVALID, "bad arguments");
  std::string out;
  for (const Group& g : B->groups) {
    char line[512];
    std::snprintf(line, sizeof(line),
                  "group instances=%d nrMax=%d nMax=%d mMax=%d %s block=%d grid=%d smem=%zu vecInSmem=%d "
                  "rootInSmem=%d root64InSmem=%d scratchPerCTA=%lld wholeGPU=%d\n",
                  g.count, g.lay.nrMax, g.lay.nMax, g.lay.mMax, g.fp32 ? "mixed" : "fp64", g.block, g.grid, g.smem,
                  g.lay.vecInSmem, g.lay.rootInSmem, g.lay.root64InSmem, (long long)g.stride, B->gridMode ? 1 : 0);
    out += line;
  }
  std::snprintf(buf, (size_t)buflen, "%s", out.c_str());
  return (int)out.size();
}

// ------------------------------------------------------------------------------------------
// autotuner: size-bucket edges, then threads per instance for each bucket, by timing whole solves
// ------------------------------------------------------------------------------------------
// Lays the per-bucket scratch regions out again after grids changed; reallocates if it grew.
static int relayoutScratch(cxg_batch* B) {
  int64_t total = 0;
  for (Group& g : B->groups) {
    g.scratchOff = total;
    total += g.stride * g.grid;
  }
  if (total > B->scratchCapacity) {
    if (B->dScratch) cudaFree(B->dScratch);
    B->dScratch = nullptr;
    B->scratchCapacity = 0;
    int rc = devAlloc(&B->dScratch, (size_t)std::max<int64_t>(total, 2));
    if (rc) return rc;
    B->scratchCapacity = std::max<int64_t>(total, 2);
  }
  return CXG_OK;
}

extern "C" int cxg_batch_autotune(cxg_batch* B, int trials, char* report, int reportLen) {
  if (!B) return setErr(CXG_E_INVALID, "null batch");
  if (B->gridMode) {  // one launch shape: a CTA of 256 threads on every SM
    if (report && reportLen > 0) std::snprintf(report, (size_t)reportLen, "whole-GPU root: nothing to tune\n");
    return CXG_OK;
  }
  if (trials < 1) trials = 1;
  int numSM = 0;
  CX_CUDA(cudaDeviceGetAttribute(&numSM, cudaDevAttrMultiProcessorCount, B->device));
  cxg_settings tst = B->st;
  tst.warm_start = 0;  // trials leave the warm-start state alone
  tst.record_timings = 0;
  const DevSettings ds = makeDevSettings(tst, B->kktSt);
  std::string rep;
  // (1) the size-bucket edges: each candidate set is planned (buckets, SM shares, scratch) and a
  //     whole concurrent solve timed; the fastest set is kept
  {
    static const std::vector<std::vector<int>> kEdgeSets = {
        {32, 64, 96, 128, 192, 256, 384, 512, 1024, 2048, 4096},
        {64, 128, 192, 256, 384, 512, 1024, 2048, 4096},
        {16, 32, 48, 64, 96, 128, 160, 192, 256, 384, 512, 1024, 2048, 4096},
        {32, 64, 128, 192, 256, 384, 512, 1024, 2048, 4096},
        {48, 96, 144, 192, 256, 384, 512, 1024, 2048, 4096}};
    const cxg_settings saved = B->st;
    B->st = tst;
    cudaEvent_t a0 = nullptr, a1 = nullptr;
    CX_CUDA(cudaEventCreate(&a0));
    CX_CUDA(cudaEventCreate(&a1));
    int best = -1, rc0 = CXG_OK;
    float bestMs = 0.0f;
    char line[160];
    for (size_t e = 0; e < kEdgeSets.size() && rc0 == CXG_OK; ++e) {
      B->edges = kEdgeSets[e];
      if ((rc0 = buildGroups(B)) || (rc0 = refreshGroupsOnDevice(B))) break;
      std::vector<float> ms;
      for (int t = 0; t < trials + 1 && rc0 == CXG_OK; ++t) {
        cudaError_t ce = cudaEventRecord(a0, B->stream);
        if (ce == cudaSuccess && (rc0 = runSolve(B, B->stream))) break;
        if (ce == cudaSuccess) ce = cudaEventRecord(a1, B->stream);
        if (ce == cudaSuccess) ce = cudaEventSynchronize(a1);
        float v = 0.0f;
        if (ce == cudaSuccess) ce = cudaEventElapsedTime(&v, a0, a1);
        if (ce != cudaSuccess) rc0 = setErr(CXG_E_CUDA, std::string("autotune: ") + cudaGetErrorString(ce));
        if (t > 0) ms.push_back(v);  // the first solve of each set captures its graph
      }
      if (rc0) break;
      std::sort(ms.begin(), ms.end());
      const float med = ms[ms.size() / 2];
      std::snprintf(line, sizeof(line), "edges set %d (%d size groups): %.3f ms\n", (int)e, (int)B->groups.size(), med);
      rep += line;
      if (best < 0 || med < bestMs) {
        best = (int)e;
        bestMs = med;
      }
    }
    cudaEventDestroy(a0);
    cudaEventDestroy(a1);
    B->st = saved;
    if (rc0) return rc0;
    B->edges = kEdgeSets[(size_t)best];
    int rcb = buildGroups(B);
    if (!rcb) rcb = refreshGroupsOnDevice(B);
    if (rcb) return rcb;
    std::snprintf(line, sizeof(line), "-> edges set %d\n", best);
    rep += line;
  }
  // (2) threads per instance for each size bucket, one bucket at a time, by timing the whole
  //     concurrent solve (the buckets share the SMs, so a shape that is faster alone can lengthen
  //     the others' time): for each candidate the SM shares and scratch are laid out again
  static const int kCand[] = {32, 64, 128, 256};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CX_CUDA(cudaEventCreate(&e0));
  CX_CUDA(cudaEventCreate(&e1));
  const cxg_settings saved = B->st;
  B->st = tst;
  int rc = CXG_OK;
  auto timeSolve = [&](float& med) -> int {
    partitionGrids(B, numSM);
    if (int r = relayoutScratch(B)) return r;
    B->graphValid = false;
    std::vector<float> ms;
    for (int t = 0; t < trials + 1; ++t) {
      cudaError_t ce = cudaEventRecord(e0, B->stream);
      if (ce == cudaSuccess)
        if (int r = runSolve(B, B->stream)) return r;
      if (ce == cudaSuccess) ce = cudaEventRecord(e1, B->stream);
      if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
      float v = 0.0f;
      if (ce == cudaSuccess) ce = cudaEventElapsedTime(&v, e0, e1);
      if (ce != cudaSuccess) return setErr(CXG_E_CUDA, std::string("autotune: ") + cudaGetErrorString(ce));
      if (t > 0) ms.push_back(v);  // the first solve of each shape captures its graph
    }
    std::sort(ms.begin(), ms.end());
    med = ms[ms.size() / 2];
    return CXG_OK;
  };
  for (size_t gi = 0; gi < B->groups.size() && rc == CXG_OK; ++gi) {
    Group& g = B->groups[gi];
    const int start = g.block;
    int bestBlock = start;
    float bestMs = 0.0f;
    char line[256];
    std::snprintf(line, sizeof(line), "bucket nr<=%d (%d instances):", g.lay.nrMax, g.count);
    rep += line;
    for (int b : kCand) {
      if (b < 64 && g.lay.nrMax > 64) continue;  // one warp only for small roots
      int occ = 0;
      if (ipmOccupancy(&occ, b, g.smem, g.fp32) != cudaSuccess || occ < 1) occ = 1;
      g.block = b;
      g.occupancy = occ;
      float med = 0.0f;
      if ((rc = timeSolve(med))) break;
      std::snprintf(line, sizeof(line), " %d threads %.3f ms;", b, med);
      rep += line;
      if (bestMs == 0.0f || med < bestMs) {
        bestMs = med;
        bestBlock = b;
      }
    }
    if (rc) break;
    g.block = bestBlock;
    {
      int occ = 0;
      if (ipmOccupancy(&occ, bestBlock, g.smem, g.fp32) != cudaSuccess || occ < 1) occ = 1;
      g.occupancy = occ;
    }
    std::snprintf(line, sizeof(line), " -> %d\n", bestBlock);
    rep += line;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  B->st = saved;
  if (rc) return rc;
  partitionGrids(B, numSM);
  if ((rc = relayoutScratch(B))) return rc;
  B->graphValid = false;  // the captured launch shapes are stale
  if (report && reportLen > 0) std::snprintf(report, (size_t)reportLen, "%s", rep.c_str());
  return CXG_OK;
}

// ------------------------------------------------------------------------------------------
// single instance (conicxx::Solver)
// ------------------------------------------------------------------------------------------
struct cxg_solver {
  cxg_batch* batch = nullptr;
  cxg_settings st{};
  bool setupDone = false;
  int n = 0, m = 0;
  std::vector<double> d, e;  // equilibration of the setup (host copy for warm-start scaling)
  double c = 1.0;
  ~cxg_solver() { delete batch; }
};

extern "C" int cxg_solver_create(cxg_solver** out) {
  if (!out) return setErr(CXG_E_INVALID, "null output handle");
  *out = new (std::nothrow) cxg_solver();
  if (!*out) return setErr(CXG_E_NOMEM, "host allocation failed");
  cxg_default_settings(&(*out)->st);
  return CXG_OK;
}

extern "C" void cxg_solver_destroy(cxg_solver* s) { delete s; }

extern "C" int cxg_solver_setup(cxg_solver* S, const cxg_problem* pr, const cxg_settings* settings) {
  if (!S || !pr) return setErr(CXG_E_INVALID, "null argument");
  S->setupDone = false;
  delete S->batch;
  S->batch = nullptr;
  cxg_settings st;
  if (settings) st = *settings;
  else {
    cxg_default_settings(&st);
    st.differentiable = 1;
  }
  S->st = st;
  // automatic whole-GPU root for a single instance: one SM factors roots up to a few hundred rows
  // in well under a millisecond, larger ones are faster spread over every SM
  cxg_settings bst = st;
  if (bst.whole_gpu_root == 0 && pr->n + pr->zero_dim > kGridAutoRoot) bst.whole_gpu_root = 1;
  int rc = cxg_batch_create(&S->batch, 1, pr, &bst);
  if (rc) return rc;
  S->n = pr->n;
  S->m = pr->m;
  const InstanceDesc& D = S->batch->pools.desc[0];
  S->d.assign(S->batch->pools.dpool.begin() + D.dD, S->batch->pools.dpool.begin() + D.dD + D.n);
  S->e.assign(S->batch->pools.dpool.begin() + D.dE, S->batch->pools.dpool.begin() + D.dE + D.m);
  S->c = D.cscale;
  S->setupDone = true;
  return CXG_OK;
}

extern "C" int cxg_solver_update_data(cxg_solver* S, const int* Pp, const int* Pi, const double* Px, const double* q,
                                      const int* Ap, const int* Ai, const double* Ax, const double* b) {
  if (!S || !S->setupDone) return setErr(CXG_E_NOT_SETUP, "updateData before setup");
  cxg_batch* B = S->batch;
  if (Px) {
    if (!Pp || !Pi) return setErr(CXG_E_INVALID, "P values given without its pattern");
    if (!samePattern(B->Pp[0], B->Pi[0], S->n, Pp, Pi)) return setErr(CXG_E_PATTERN, "P sparsity pattern changed");
    std::string e = checkFinite(Px, Pp[S->n], "P");
    if (!e.empty()) return setErr(CXG_E_INVALID, e);
  }
  if (Ax) {
    if (!Ap || !Ai) return setErr(CXG_E_INVALID, "A values given without its pattern");
    if (!samePattern(B->Ap[0], B->Ai[0], S->n, Ap, Ai)) return setErr(CXG_E_PATTERN, "A sparsity pattern changed");
    std::string e = checkFinite(Ax, Ap[S->n], "A");
    if (!e.empty()) return setErr(CXG_E_INVALID, e);
  }
  if (q) { std::string e = checkFinite(q, S->n, "q"); if (!e.empty()) return setErr(CXG_E_INVALID, e); }
  if (b) { std::string e = checkFinite(b, S->m, "b"); if (!e.empty()) return setErr(CXG_E_INVALID, e); }
  return cxg_batch_update_values(B, Px, q, Ax, b);
}

extern "C" int cxg_solver_set_warm_start(cxg_solver* S, const double* x, const double* s, const double* z) {
  if (!S || !S->setupDone) return CXG_OK;  // the reference silently ignores it before setup
  if (!x || !s || !z) return setErr(CXG_E_INVALID, "null warm-start vector");
  cxg_batch* B = S->batch;
  const bool eq = B->kktSt.equilibrate != 0;
  std::vector<double> wx(x, x + S->n), ws(s, s + S->m), wz(z, z + S->m);
  if (eq) {  // equilibration.cpp:135-139
    for (int i = 0; i < S->n; ++i) wx[(size_t)i] /= S->d[(size_t)i];
    for (int i = 0; i < S->m; ++i) {
      wz[(size_t)i] = wz[(size_t)i] * S->c / S->e[(size_t)i];
      ws[(size_t)i] *= S->e[(size_t)i];
    }
  }
  CX_CUDA(cudaMemcpy(B->dWx, wx.data(), sizeof(double) * wx.size(), cudaMemcpyHostToDevice));
  if (S->m) {
    CX_CUDA(cudaMemcpy(B->dWs, ws.data(), sizeof(double) * ws.size(), cudaMemcpyHostToDevice));
    CX_CUDA(cudaMemcpy(B->dWz, wz.data(), sizeof(double) * wz.size(), cudaMemcpyHostToDevice));
  }
  const unsigned char one = 1;
  CX_CUDA(cudaMemcpy(B->dHaveWarm, &one, 1, cudaMemcpyHostToDevice));
  return CXG_OK;
}

extern "C" int cxg_solver_set_settings(cxg_solver* S, const cxg_settings* st) {
  if (!S || !st) return setErr(CXG_E_INVALID, "null argument");
  S->st = *st;
  if (S->batch) S->batch->st = *st;  // KKT fields stay as frozen at setup (kkt_system.cpp:26-31)
  return CXG_OK;
}

extern "C" int cxg_solver_get_settings(const cxg_solver* S, cxg_settings* out) {
  if (!S || !out) return setErr(CXG_E_INVALID, "null argument");
  *out = S->st;
  return CXG_OK;
}

extern "C" int cxg_solver_solve(cxg_solver* S, double* x, double* s, double* z, cxg_info* info) {
  if (!S) return setErr(CXG_E_INVALID, "null solver");
  if (!S->setupDone) {  // solver_impl.cpp:369-372 of the reference: NumericalError before setup
    if (info) {
      std::memset(info, 0, sizeof(*info));
      info->status = CXG_STATUS_NUMERICAL_ERROR;
    }
    return CXG_OK;
  }
  return cxg_batch_solve(S->batch, x, s, z, info);
}

extern "C" int cxg_solver_backward(cxg_solver* S, const double* dL_dx, double* dq, double* db, double* dPx, double* dAx) {
  if (!S || !S->setupDone) return setErr(CXG_E_NOT_SETUP, "backward before setup");
  return cxg_batch_backward(S->batch, dL_dx, dq, db, dPx, dAx);
}

extern "C" int cxg_batch_backward(cxg_batch* B, const double* dL_dx, double* dq, double* db, double* dPx, double* dAx);

// Enqueues the adjoint of every instance (one launch per size bucket, forked like the solve).
static int enqueueAdjoint(cxg_batch* B, cudaStream_t s, const double* gx, double* gq, double* gb, double* gP,
                          double* gA) {
  const DevSettings ds = makeDevSettings(B->st, B->kktSt);
  CX_CUDA(cudaMemsetAsync(B->dCounters, 0, sizeof(int) * (B->groups.size() + 1), s));
  const size_t G = B->groups.size();
  CX_CUDA(cudaEventRecord(B->forkJoin[0], s));
  // Launch order: by shared memory per CTA, largest first. The grids are apportioned so that all
  // of them can be resident at once (partitionGrids); the block scheduler spreads each launch's
  // CTAs over the SMs with room left, so the largest CTAs must be placed before the small ones
  // scatter over every SM and leave no SM with room for a large one (first fit, decreasing).
  std::vector<size_t> launchOrder(G);
  std::iota(launchOrder.begin(), launchOrder.end(), size_t(0));
  std::stable_sort(launchOrder.begin(), launchOrder.end(),
                   [&](size_t a_, size_t b_) { return B->groups[a_].smem > B->groups[b_].smem; });
  for (size_t rank = 0; rank < G; ++rank) {
    const size_t gi = launchOrder[rank];
    const Group& g = B->groups[gi];
    cudaStream_t gs = (G == 1) ? s : B->groupStreams[rank];
    if (G > 1) CX_CUDA(cudaStreamWaitEvent(gs, B->forkJoin[0], 0));
    LaunchArgs a{};
    a.desc = B->dDesc;
    a.order = B->dOrder + g.begin;
    a.count = g.count;
    a.counter = B->dCounters + g.counterIdx;
    a.ipool = B->dIpool;
    a.dpool = B->dDpool;
    a.Px = B->dPx;
    a.q = B->dq;
    a.Ax = B->dAx;
    a.b = B->db;
    a.bwd = B->dBwd;
    a.gx = gx;
    a.gq = gq;
    a.gb = gb;
    a.gP = gP;
    a.gA = gA;
    a.scratch = B->dScratch + g.scratchOff;
    a.scratchStride = g.stride;
    a.st = ds;
    a.lay = g.lay;
    // whole-GPU form: the single instance and its scratch belong to CTA 0 (one CTA)
    CX_CUDA(launchAdjoint(a, B->gridMode ? 1 : g.grid, g.block, g.smem, gs));
    if (G > 1) {
      CX_CUDA(cudaEventRecord(B->forkJoin[gi + 1], gs));
      CX_CUDA(cudaStreamWaitEvent(s, B->forkJoin[gi + 1], 0));
    }
  }
  B->lastLaunches = (int)G;
  return CXG_OK;
}

static int checkDifferentiable(cxg_batch* B) {
  if (!B) return setErr(CXG_E_INVALID, "null batch");
  if (!B->dBwd && B->bwdDropped)
    return setErr(CXG_E_UNSUPPORTED, "backward is offered up to 8192 root rows on the whole-GPU root");
  if (!B->dBwd) return setErr(CXG_E_NOT_SETUP, "backward needs settings.differentiable = 1 at set-up");
  if (B->forkJoin.empty()) return setErr(CXG_E_NOT_SETUP, "backward before any solve");
  if (B->bwdStale) return setErr(CXG_E_NOT_SETUP, "backward after cxg_batch_replace needs a solve first");
  return CXG_OK;
}

extern "C" int cxg_batch_backward(cxg_batch* B, const double* dL_dx, double* dq, double* db, double* dPx, double* dAx) {
  int rc = checkDifferentiable(B);
  if (rc) return rc;
  if (!dL_dx) return setErr(CXG_E_INVALID, "null dL/dx");
  CX_CUDA(cudaMemcpyAsync(B->dGx, dL_dx, (size_t)B->pools.totQ * 8, cudaMemcpyHostToDevice, B->stream));
  rc = enqueueAdjoint(B, B->stream, B->dGx, B->dGq, B->dGb, B->dGP, B->dGA);
  if (rc) return rc;
  if (dq && B->pools.totQ) CX_CUDA(cudaMemcpyAsync(dq, B->dGq, (size_t)B->pools.totQ * 8, cudaMemcpyDeviceToHost, B->stream));
  if (db && B->pools.totB) CX_CUDA(cudaMemcpyAsync(db, B->dGb, (size_t)B->pools.totB * 8, cudaMemcpyDeviceToHost, B->stream));
  if (dPx && B->pools.totPx) CX_CUDA(cudaMemcpyAsync(dPx, B->dGP, (size_t)B->pools.totPx * 8, cudaMemcpyDeviceToHost, B->stream));
  if (dAx && B->pools.totAx) CX_CUDA(cudaMemcpyAsync(dAx, B->dGA, (size_t)B->pools.totAx * 8, cudaMemcpyDeviceToHost, B->stream));
  CX_CUDA(cudaStreamSynchronize(B->stream));
  return CXG_OK;
}

extern "C" int cxg_batch_backward_device(cxg_batch* B, const double* dL_dx, double* dq, double* db, double* dPx,
                                         double* dAx, void* stream) {
  int rc = checkDifferentiable(B);
  if (rc) return rc;
  if (!dL_dx) return setErr(CXG_E_INVALID, "null dL/dx");
  return enqueueAdjoint(B, (cudaStream_t)stream, dL_dx, dq ? dq : B->dGq, db ? db : B->dGb, dPx ? dPx : B->dGP,
                        dAx ? dAx : B->dGA);
}

// ------------------------------------------------------------------------------------------
// allocation-free solve (no reference counterpart)
// ------------------------------------------------------------------------------------------
// Some callers cannot allocate or free device memory while they solve. An example is a
// simulator's per-timestep loop that reserved its memory up front: there an allocation may fail
// mid-step and cudaFree synchronises the device. For them the IPM kernel's per-CTA working memory
// comes from this fixed array instead of the batch's own scratch.
//
// Layout: the first kNoallocCounterBytes hold the work-queue counters (one int per size bucket).
// These must be zero when a launch starts, so every call clears them on its stream. The rest is
// the per-CTA FP64 scratch. The kernel writes scratch before it reads it, so no clearing is needed.
static __device__ __align__(256) unsigned char g_noallocArena[CXG_NOALLOC_SCRATCH_BYTES];
constexpr int64_t kNoallocCounterBytes = 256;
constexpr int kNoallocMaxDevices = 64;
static unsigned char* g_noallocPtr[kNoallocMaxDevices];
static std::mutex g_noallocMutex;

// Address of the array on the current device `dev`. It is looked up once per device, on the first
// call with that device current; that lookup loads this module if it is not loaded yet.
static int noallocArena(int dev, unsigned char** out) {
  if (dev < 0 || dev >= kNoallocMaxDevices) return setErr(CXG_E_UNSUPPORTED, "device index beyond 63");
  std::lock_guard<std::mutex> lock(g_noallocMutex);
  if (!g_noallocPtr[dev]) {
    unsigned char* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noallocArena);
    if (e != cudaSuccess || !ptr)
      return setErr(CXG_E_CUDA, std::string("cudaGetSymbolAddress(fixed scratch): ") + cudaGetErrorString(e));
    g_noallocPtr[dev] = ptr;
  }
  *out = g_noallocPtr[dev];
  return CXG_OK;
}

extern "C" int cxg_batch_solve_device_noalloc(cxg_batch* B, double* x, double* s, double* z, cxg_info* info,
                                              void* stream) {
  if (!B) return setErr(CXG_E_INVALID, "null batch");
  if (B->gridMode) return setErr(CXG_E_UNSUPPORTED, "the whole-GPU root of a single large instance has its own scratch");
  B->bwdStale = false;
  int dev = -1;
  CX_CUDA(cudaGetDevice(&dev));
  if (dev != B->device) return setErr(CXG_E_INVALID, "the batch lives on another device: make that device current");
  const size_t G = B->groups.size();
  if ((int64_t)(G * sizeof(int)) > kNoallocCounterBytes) return setErr(CXG_E_INTERNAL, "too many size buckets");
  const int64_t capDoubles = (CXG_NOALLOC_SCRATCH_BYTES - kNoallocCounterBytes) / (int64_t)sizeof(double);
  for (const Group& g : B->groups)
    if (g.stride > capDoubles) {
      char msg[256];
      std::snprintf(msg, sizeof(msg),
                    "an instance of this batch needs %lld bytes of working memory per CTA (bucket nr <= %d); "
                    "the fixed scratch holds %lld",
                    (long long)(g.stride * 8), g.lay.nrMax, (long long)(capDoubles * 8));
      return setErr(CXG_E_UNSUPPORTED, msg);
    }
  unsigned char* arena = nullptr;
  int rc = noallocArena(dev, &arena);
  if (rc) return rc;
  int* counters = (int*)arena;
  double* scratch = (double*)(arena + kNoallocCounterBytes);
  cudaStream_t st = (cudaStream_t)stream;
  CX_CUDA(cudaMemsetAsync(counters, 0, (size_t)kNoallocCounterBytes, st));
  const DevSettings ds = makeDevSettings(B->st, B->kktSt);
  // Buckets run in stream order, so each may use the whole scratch from its start.
  for (size_t gi = 0; gi < G; ++gi) {
    const Group& g = B->groups[gi];
    LaunchArgs a{};
    a.desc = B->dDesc;
    a.order = B->dOrder + g.begin;
    a.count = g.count;
    a.counter = counters + gi;
    a.ipool = B->dIpool;
    a.dpool = B->dDpool;
    a.Px = B->dPx;
    a.q = B->dq;
    a.Ax = B->dAx;
    a.b = B->db;
    a.x = B->dx;
    a.s = B->ds;
    a.z = B->dz;
    a.results = B->dRes;
    a.warmX = B->dWx;
    a.warmS = B->dWs;
    a.warmZ = B->dWz;
    a.haveWarm = B->dHaveWarm;
    a.bwd = B->dBwd;
    a.scratch = scratch;
    a.scratchStride = g.stride;
    a.st = ds;
    a.lay = g.lay;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(g.gridAlone, capDoubles / g.stride));
    CX_CUDA(launchIpm(a, grid, g.block, g.smem, g.fp32, st));
  }
  // history-ordered queues for the next solve, as the other solve entry points keep them (the
  // re-ordering kernel uses static shared memory and the batch's own queue array only)
  rc = enqueueReorder(B, st);
  if (rc) return rc;
  B->lastLaunches = (int)G + ((G >= 1 && G <= (size_t)kMaxGroups) ? 1 : 0);
  if (x && B->pools.totQ) CX_CUDA(cudaMemcpyAsync(x, B->dx, (size_t)B->pools.totQ * 8, cudaMemcpyDeviceToDevice, st));
  if (s && B->pools.totB) CX_CUDA(cudaMemcpyAsync(s, B->ds, (size_t)B->pools.totB * 8, cudaMemcpyDeviceToDevice, st));
  if (z && B->pools.totB) CX_CUDA(cudaMemcpyAsync(z, B->dz, (size_t)B->pools.totB * 8, cudaMemcpyDeviceToDevice, st));
  if (info) {
    CX_CUDA(cudaStreamSynchronize(st));
    return fetchInfo(B, info, 0.0);
  }
  return CXG_OK;
}

static int traceCopy(cxg_batch* B, int instance, double* out, int capRows) {
  if (!B || !out || capRows < 0) return setErr(CXG_E_INVALID, "null argument");
  if (instance < 0 || instance >= B->count) return setErr(CXG_E_INVALID, "instance index out of range");
  if (!B->dTrace) return setErr(CXG_E_INVALID, "no trace: solve with record_timings set first");
  DevResult R{};
  CX_CUDA(cudaMemcpy(&R, B->dRes + instance, sizeof(DevResult), cudaMemcpyDeviceToHost));
  const int rows = std::min({R.iterations, B->traceRows, capRows});
  if (rows > 0)
    CX_CUDA(cudaMemcpy(out, B->dTrace + (size_t)instance * B->traceRows * kTraceCols,
                       sizeof(double) * (size_t)rows * kTraceCols, cudaMemcpyDeviceToHost));
  return rows;
}

extern "C" int cxg_batch_trace(cxg_batch* B, int instance, double* out, int cap_rows) {
  return traceCopy(B, instance, out, cap_rows);
}

extern "C" int cxg_solver_trace(cxg_solver* S, double* out, int cap_rows) {
  if (!S || !S->setupDone || !S->batch) return setErr(CXG_E_INVALID, "solver not set up");
  return traceCopy(S->batch, 0, out, cap_rows);
}

// Batched solves and the tile autotuner of the GB300 DG path (sdg_batch_*, sdg_autotune, sdg_*_tile).
//
// A batch turns the launch records of every instance's step (sdg_internal.hpp: emitStep) into one
// persistent launch per (dependency level, kernel variant, tile shape): the records' argument blocks go
// to a device table, and a work list of (argument index, tile or point chunk) items spans all instances.
// Launches of one level are independent (they touch disjoint instances or disjoint slots of one
// instance) and run on forked streams; the whole step is captured once into a CUDA graph.  The
// persistent CTAs stride over the work list, so small instances (a few hundred elements, one or two
// tiles each) share the GPU instead of each leaving most of its SMs idle.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>

#include "sdg_internal.hpp"

using namespace sdg;

namespace {

struct Group {
  int seq = 0, kind = 0;
  const void* bfn = nullptr;
  int threads = 0, epb = 0;
  size_t smem = 0;
  std::vector<int> recs;           // indices into the batch's record list
  void* dArgs = nullptr;           // argument table [nargs]
  Phys* dPhys = nullptr;           // stage kernels: physics per argument set
  int2* dItems = nullptr;          // work list [nitems]
  int nitems = 0, nargs = 0;
  int grid = 0;
  size_t argBytes = 0;
};

size_t argSize(int kind) {
  switch (kind) {
    case kRecStage: return sizeof(StageArgs);
    case kRecGradTensor: return sizeof(GradArgs);
    case kRecGradDense: return sizeof(DenseGradArgs);
    case kRecFace: return sizeof(FaceArgs);
    case kRecAv: return sizeof(AvArgs);
    default: return sizeof(RelArgs);
  }
}

const void* argPtr(const Rec& r) {
  switch (r.kind) {
    case kRecStage: return &r.sa;
    case kRecGradTensor: return &r.ga;
    case kRecGradDense: return &r.da;
    case kRecFace: return &r.fa;
    case kRecAv: return &r.av;
    default: return &r.ra;
  }
}

// Process-wide tile cache: (device, kernel, size class) -> (elements per CTA, threads).
std::mutex g_tune_mutex;
std::map<std::tuple<int, const void*, int>, std::pair<int, int>> g_tune;

int sizeClass(int64_t ne) {
  int c = 0;
  while ((int64_t(1) << (c + 1)) <= ne && c < 40) ++c;
  return c;
}

}  // namespace

struct sdg_batch {
  int device = 0;
  bool planOnly = false;
  cudaStream_t stream = nullptr;
  std::vector<cudaStream_t> side;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  std::vector<sdg_handle*> inst;
  std::vector<double> dt;
  bool haveDt = false;
  std::vector<Rec> recs;
  std::vector<Group> groups;       // execution order (by level)
  int persist = 2;                 // persistent CTAs per SM (0: one CTA per work item)
  cudaGraphExec_t exec = nullptr;
  bool built = false;
  int64_t items = 0;
  int stages = 0;
  int sequentialLaunches = 0;
  std::vector<std::vector<Rec>> seqRecs;  // per instance, for the sequential baseline
  std::string err;
};

namespace {

constexpr int kSideStreams = 4;

void freeGroups(sdg_batch* b) {
  for (Group& g : b->groups) {
    cudaFree(g.dArgs); cudaFree(g.dPhys); cudaFree(g.dItems);
  }
  b->groups.clear();
}

void dropExec(sdg_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
}

void emitAll(sdg_batch* b) {
  b->recs.clear();
  b->seqRecs.assign(b->inst.size(), {});
  b->stages = 0;
  for (size_t i = 0; i < b->inst.size(); ++i) {
    sdg_handle* h = b->inst[i];
    emitStep(h, b->haveDt ? b->dt[i] : 0.0, true, b->seqRecs[i]);
    b->stages = std::max(b->stages, h->cfg.time_integration + 1);
    b->recs.insert(b->recs.end(), b->seqRecs[i].begin(), b->seqRecs[i].end());
  }
  b->sequentialLaunches = 0;
  for (const Rec& r : b->recs) b->sequentialLaunches += r.units > 0;
}

// Host argument table and work list of a group.
void groupTables(const sdg_batch* b, const Group& g, std::vector<unsigned char>& args, std::vector<Phys>& phys,
                 std::vector<int2>& items) {
  const size_t sz = argSize(g.kind);
  args.assign(sz * g.recs.size(), 0);
  phys.clear();
  items.clear();
  for (size_t k = 0; k < g.recs.size(); ++k) {
    const Rec& r = b->recs[g.recs[k]];
    std::memcpy(args.data() + k * sz, argPtr(r), sz);
    phys.push_back(r.ph);
    if (g.kind == kRecRelerr) continue;
    for (int64_t t = 0; t < r.units; ++t) items.push_back(make_int2(int(k), int(t)));
  }
}

int persistentGrid(const sdg_batch* b, const Group& g) {
  if (g.kind == kRecRelerr) return g.nargs;
  if (b->persist <= 0 || b->planOnly) return g.nitems;
  int occ = 0;
  SDG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, g.bfn, g.threads, g.smem));
  occ = std::max(1, std::min(occ, b->persist));
  const int64_t cap = int64_t(occ) * multiprocessorCount(b->device);
  return int(std::min<int64_t>(g.nitems, cap));
}

void build(sdg_batch* b) {
  dropExec(b);
  freeGroups(b);
  emitAll(b);
  std::map<std::tuple<int, const void*, int, int, size_t>, int> index;
  for (size_t i = 0; i < b->recs.size(); ++i) {
    const Rec& r = b->recs[i];
    if (r.units <= 0) continue;
    const auto key = std::make_tuple(r.seq, r.bfn, r.threads, r.epb, r.smem);
    auto it = index.find(key);
    if (it == index.end()) {
      Group g;
      g.seq = r.seq; g.kind = r.kind; g.bfn = r.bfn; g.threads = r.threads; g.epb = r.epb; g.smem = r.smem;
      it = index.emplace(key, int(b->groups.size())).first;
      b->groups.push_back(g);
    }
    b->groups[it->second].recs.push_back(int(i));
  }
  std::stable_sort(b->groups.begin(), b->groups.end(), [](const Group& x, const Group& y) { return x.seq < y.seq; });
  b->items = 0;
  std::vector<unsigned char> args;
  std::vector<Phys> phys;
  std::vector<int2> items;
  for (Group& g : b->groups) {
    groupTables(b, g, args, phys, items);
    g.nargs = int(g.recs.size());
    g.nitems = g.kind == kRecRelerr ? g.nargs : int(items.size());
    g.argBytes = args.size();
    b->items += g.nitems;
    if (!b->planOnly) {
      SDG_CUDA(cudaMalloc(&g.dArgs, std::max<size_t>(args.size(), 16)));
      SDG_CUDA(cudaMemcpyAsync(g.dArgs, args.data(), args.size(), cudaMemcpyHostToDevice, b->stream));
      if (g.kind == kRecStage) {
        SDG_CUDA(cudaMalloc(reinterpret_cast<void**>(&g.dPhys), phys.size() * sizeof(Phys)));
        SDG_CUDA(cudaMemcpyAsync(g.dPhys, phys.data(), phys.size() * sizeof(Phys), cudaMemcpyHostToDevice, b->stream));
      }
      if (!items.empty()) {
        SDG_CUDA(cudaMalloc(reinterpret_cast<void**>(&g.dItems), items.size() * sizeof(int2)));
        SDG_CUDA(cudaMemcpyAsync(g.dItems, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
      }
    }
    g.grid = persistentGrid(b, g);
  }
  if (!b->planOnly) SDG_CUDA(cudaStreamSynchronize(b->stream));
  b->built = true;
}

// New dt: rewrite the argument tables in place (the graph keeps the same device pointers).
void refreshArgs(sdg_batch* b) {
  emitAll(b);
  std::vector<unsigned char> args;
  std::vector<Phys> phys;
  std::vector<int2> items;
  for (Group& g : b->groups) {
    if (g.kind != kRecStage) continue;
    // the records of a group are found again by position: emitAll produces the same order
    groupTables(b, g, args, phys, items);
    SDG_CUDA(cudaMemcpyAsync(g.dArgs, args.data(), args.size(), cudaMemcpyHostToDevice, b->stream));
  }
  SDG_CUDA(cudaStreamSynchronize(b->stream));
}

void launchGroup(const Group& g, cudaStream_t s) {
  void* dArgs = g.dArgs;
  void* dPhys = g.dPhys;
  void* dItems = g.dItems;
  int nitems = g.nitems, epb = g.epb;
  void* p5[5] = {&dArgs, &dPhys, &dItems, &nitems, &epb};
  void* p4[4] = {&dArgs, &dItems, &nitems, &epb};
  void* p3[3] = {&dArgs, &dItems, &nitems};
  void* p1[1] = {&dArgs};
  switch (g.kind) {
    case kRecStage: SDG_CUDA(cudaLaunchKernel(g.bfn, dim3(g.grid), dim3(g.threads), p5, g.smem, s)); break;
    case kRecGradTensor:
    case kRecGradDense: SDG_CUDA(cudaLaunchKernel(g.bfn, dim3(g.grid), dim3(g.threads), p4, g.smem, s)); break;
    case kRecFace:
    case kRecAv: SDG_CUDA(cudaLaunchKernel(g.bfn, dim3(g.grid), dim3(g.threads), p3, g.smem, s)); break;
    default: SDG_CUDA(cudaLaunchKernel(g.bfn, dim3(5, g.grid), dim3(g.threads), p1, 0, s)); break;
  }
}

void capture(sdg_batch* b) {
  dropExec(b);
  cudaGraph_t graph = nullptr;
  SDG_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  try {
    size_t i = 0;
    while (i < b->groups.size()) {
      size_t j = i;
      while (j < b->groups.size() && b->groups[j].seq == b->groups[i].seq) ++j;
      if (j - i == 1) {
        launchGroup(b->groups[i], b->stream);
      } else {
        SDG_CUDA(cudaEventRecord(b->fork, b->stream));
        const size_t used = std::min<size_t>(j - i, b->side.size());
        for (size_t k = 0; k < used; ++k) SDG_CUDA(cudaStreamWaitEvent(b->side[k], b->fork, 0));
        for (size_t k = i; k < j; ++k) launchGroup(b->groups[k], b->side[(k - i) % b->side.size()]);
        for (size_t k = 0; k < used; ++k) {
          SDG_CUDA(cudaEventRecord(b->join[k], b->side[k]));
          SDG_CUDA(cudaStreamWaitEvent(b->stream, b->join[k], 0));
        }
      }
      i = j;
    }
  } catch (...) {
    cudaStreamEndCapture(b->stream, &graph);
    if (graph) cudaGraphDestroy(graph);
    throw;
  }
  SDG_CUDA(cudaStreamEndCapture(b->stream, &graph));
  const cudaError_t e = cudaGraphInstantiate(&b->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) { b->exec = nullptr; SDG_CUDA(e); }
}

void ready(sdg_batch* b) {
  if (b->planOnly) throw Failure(SDG_ERR_STATE, "the batch holds host-only instances: it can only plan");
  if (!b->haveDt) throw Failure(SDG_ERR_STATE, "sdg_batch_set_delta_time before the first step");
  for (sdg_handle* h : b->inst)
    if (!h->hasState) throw Failure(SDG_ERR_STATE, "every instance needs an initial state");
  if (!b->built) build(b);
  if (!b->exec) capture(b);
}

void stepBatch(sdg_batch* b, int steps) {
  ready(b);
  for (sdg_handle* h : b->inst) h->stateVersion++;
  for (int s = 0; s < steps; ++s) SDG_CUDA(cudaGraphLaunch(b->exec, b->stream));
}

// ---- autotuner -------------------------------------------------------------------------------------
float timeLaunches(const std::vector<Rec>& recs, sdg_handle* h, int reps) {
  cudaEvent_t e0, e1;
  SDG_CUDA(cudaEventCreate(&e0));
  SDG_CUDA(cudaEventCreate(&e1));
  const std::vector<Rec> list(recs);
  runRecs(h, list, h->stream);  // warm-up
  SDG_CUDA(cudaEventRecord(e0, h->stream));
  for (int k = 0; k < reps; ++k) runRecs(h, list, h->stream);
  SDG_CUDA(cudaEventRecord(e1, h->stream));
  SDG_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  SDG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms / float(reps);
}

// Stage kernel of block B as a timing probe: reads state[0] and the face buffer, writes state[1] only.
Rec stageProbe(sdg_handle* h, DevBlock& B) {
  Rec r = stageRec(h, B);
  r.sa.uin = h->state[0] + B.stateOffset;
  r.sa.ubase = h->state[0] + B.stateOffset;
  r.sa.uout = h->state[1] + B.stateOffset;
  r.sa.c0 = 0.0; r.sa.c1 = 1.0; r.sa.c2dt = 0.0;
  r.sa.doUpdate = 1; r.sa.doTrace = 0; r.sa.doVolume = 1;
  return r;
}

struct Candidate { int epb, threads; };

std::vector<Candidate> candidates(const KernelVariant& v, int64_t ne, int optin) {
  std::vector<Candidate> out;
  static const int kEpb[] = {1, 2, 3, 4, 5, 6, 8, 10, 12, 16, 20, 24, 32, 40, 48, 64};
  static const int kThreads[] = {64, 128, 256, 512};
  for (int e : kEpb) {
    if (e > std::max<int64_t>(1, ne)) break;
    if (v.nodeThreads) {
      const int t = v.threadsFor(e);
      if (t <= kMaxThreads && v.smem(e, t) <= size_t(optin)) out.push_back({e, t});
    } else {
      for (int t : kThreads)
        if (v.smem(e, t) <= size_t(optin)) out.push_back({e, t});
    }
  }
  return out;
}

// Tune one kernel of block B; `stage` selects the stage kernel, else the gradient kernel.
void tuneKernel(sdg_handle* h, DevBlock& B, bool stage, bool retime) {
  const KernelVariant& v = stage ? B.stageV[stageSlot(h)] : B.gradV;
  const auto key = std::make_tuple(h->device, v.single, sizeClass(B.ne));
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tune.find(key);
    if (it != g_tune.end() && !retime) {
      if (stage) setStageTile(B, stageSlot(h), it->second.first, it->second.second);
      else setGradTile(B, it->second.first, it->second.second);
      return;
    }
  }
  const int optin = sharedMemoryOptin(h->device);
  float best = 1e30f;
  Candidate pick{stage ? B.epb : B.gepb, stage ? B.threads : B.gthreads};
  for (const Candidate& c : candidates(v, B.ne, optin)) {
    if (stage) setStageTile(B, stageSlot(h), c.epb, c.threads);
    else setGradTile(B, c.epb, c.threads);
    const Rec r = stage ? stageProbe(h, B) : gradRec(h, B, 0);
    // repetitions: about 2 ms of work per candidate, at least 3
    const float one = timeLaunches({r}, h, 1);
    const int reps = std::max(3, std::min(200, int(2.0f / std::max(one, 1e-3f))));
    const float t = timeLaunches({r}, h, reps);
    if (t < best) { best = t; pick = c; }
  }
  if (stage) setStageTile(B, stageSlot(h), pick.epb, pick.threads);
  else setGradTile(B, pick.epb, pick.threads);
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  g_tune[key] = {pick.epb, pick.threads};
}

void autotune(sdg_handle* h, int flags) {
  if (h->hostOnly) throw Failure(SDG_ERR_STATE, "host-only handle (created with device < 0)");
  if (!h->hasState) throw Failure(SDG_ERR_STATE, "autotuning needs a state");
  SDG_CUDA(cudaSetDevice(h->device));
  const bool timing = h->timing;
  h->timing = false;
  const int64_t launches = h->launches;
  for (DevBlock& B : h->blocks) {
    tuneKernel(h, B, true, flags & SDG_AUTOTUNE_RETIME);
    if (viscousPath(h)) tuneKernel(h, B, false, flags & SDG_AUTOTUNE_RETIME);
  }
  h->timing = timing;
  h->launches = launches;  // probes are not the solver's launches
  dropGraph(h);
  checkStatus(h);
}

int batchFail(sdg_batch* b, const Failure& f) {
  if (b) b->err = f.what();
  return f.code;
}

}  // namespace

#pragma GCC visibility push(default)
extern "C" {

int sdg_set_graph(sdg_handle* h, int32_t enable) {
  if (!h) return SDG_ERR_INVALID_ARGUMENT;
  h->useGraph = enable != 0;
  if (!h->useGraph) dropGraph(h);
  return SDG_OK;
}

int sdg_set_wait_check(sdg_handle* h, uint32_t wait_limit, uint32_t extra_expected_bytes) {
  if (!h || extra_expected_bytes > 65536) return SDG_ERR_INVALID_ARGUMENT;
  h->waitLimit = wait_limit;
  h->txExtra = extra_expected_bytes;
  dropGraph(h);
  return SDG_OK;
}

int sdg_get_tile(const sdg_handle* h, int32_t block, int32_t* epb, int32_t* threads, int32_t* gepb, int32_t* gthreads) {
  if (!h || block < 0 || block >= int32_t(h->blocks.size())) return SDG_ERR_INVALID_ARGUMENT;
  const DevBlock& B = h->blocks[block];
  if (epb) *epb = B.epb;
  if (threads) *threads = B.threads;
  if (gepb) *gepb = B.gepb;
  if (gthreads) *gthreads = B.gthreads;
  return SDG_OK;
}

int sdg_set_tile(sdg_handle* h, int32_t block, int32_t epb, int32_t threads, int32_t gepb, int32_t gthreads) {
  if (!h || block < 0 || block >= int32_t(h->blocks.size())) return SDG_ERR_INVALID_ARGUMENT;
  DevBlock& B = h->blocks[block];
  try {
    const int limit = h->hostOnly ? 232448 : sharedMemoryOptin(h->device);  // 227 KB: the sm_103 opt-in limit
    const auto check = [&](const KernelVariant& v, int e, int t) {
      if (e < 1 || e > 1024) return false;
      const int tt = v.nodeThreads ? v.threadsFor(e) : t;
      return tt >= 32 && tt <= kMaxThreads && tt % 32 == 0 && v.smem(e, tt) <= size_t(limit);
    };
    if (!check(B.stageV[stageSlot(h)], epb, threads) || !check(B.gradV, gepb, gthreads)) {
      h->err = "tile outside the kernel's limits (threads 32..512 in whole warps, shared memory)";
      return SDG_ERR_INVALID_ARGUMENT;
    }
    setStageTile(B, stageSlot(h), epb, threads);
    setGradTile(B, gepb, gthreads);
    dropGraph(h);
  } catch (const Failure& f) {
    h->err = f.what();
    return f.code;
  }
  return SDG_OK;
}

int sdg_autotune(sdg_handle* h, int32_t flags) {
  if (!h) return SDG_ERR_INVALID_ARGUMENT;
  try {
    autotune(h, flags);
  } catch (const Failure& f) {
    h->err = f.what();
    return f.code;
  }
  return SDG_OK;
}

const char* sdg_batch_last_error(const sdg_batch* b) { return b ? b->err.c_str() : "null batch"; }

int sdg_batch_create(sdg_handle* const* instances, int32_t count, sdg_batch** out) {
  if (!instances || count <= 0 || !out) return SDG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  std::unique_ptr<sdg_batch> B(new sdg_batch());
  sdg_batch* b = B.get();
  for (int32_t i = 0; i < count; ++i) {
    if (!instances[i]) return SDG_ERR_INVALID_ARGUMENT;
    b->inst.push_back(instances[i]);
  }
  b->planOnly = b->inst[0]->hostOnly;
  b->device = b->inst[0]->device;
  for (sdg_handle* h : b->inst)
    if (h->hostOnly != b->planOnly || (!h->hostOnly && h->device != b->device)) return SDG_ERR_INVALID_ARGUMENT;
  for (size_t i = 0; i < b->inst.size(); ++i)
    for (size_t j = 0; j < i; ++j)
      if (b->inst[i] == b->inst[j]) return SDG_ERR_INVALID_ARGUMENT;  // an instance appears once
  try {
    if (!b->planOnly) {
      SDG_CUDA(cudaSetDevice(b->device));
      SDG_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
      b->side.resize(kSideStreams);
      b->join.resize(kSideStreams);
      for (int k = 0; k < kSideStreams; ++k) {
        SDG_CUDA(cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking));
        SDG_CUDA(cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming));
      }
      SDG_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    }
    b->dt.assign(b->inst.size(), 0.0);
    build(b);
  } catch (const Failure& f) {
    sdg::setCreateError(f.what());
    sdg_batch_destroy(B.release());
    return f.code;
  }
  *out = B.release();
  return SDG_OK;
}

int sdg_batch_destroy(sdg_batch* b) {
  if (!b) return SDG_ERR_INVALID_ARGUMENT;
  if (!b->planOnly) {
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
  }
  dropExec(b);
  freeGroups(b);
  for (cudaStream_t s : b->side) if (s) cudaStreamDestroy(s);
  for (cudaEvent_t e : b->join) if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return SDG_OK;
}

int sdg_batch_get_counts(const sdg_batch* b, sdg_batch_counts* c) {
  if (!b || !c) return SDG_ERR_INVALID_ARGUMENT;
  std::memset(c, 0, sizeof(*c));
  c->instance_count = int32_t(b->inst.size());
  c->launches_per_step = int32_t(b->groups.size());
  c->sequential_launches_per_step = b->sequentialLaunches;
  c->persistent_ctas_per_sm = b->persist;
  c->work_items_per_step = b->items;
  for (const sdg_handle* h : b->inst) { c->element_count += h->elements; c->degree_of_freedom_count += h->dof; }
  c->stage_count = b->stages;
  return SDG_OK;
}

int sdg_batch_set_delta_time(sdg_batch* b, const double* dt) {
  if (!b || !dt) return SDG_ERR_INVALID_ARGUMENT;
  for (size_t i = 0; i < b->inst.size(); ++i)
    if (!std::isfinite(dt[i])) return SDG_ERR_INVALID_ARGUMENT;
  try {
    b->dt.assign(dt, dt + b->inst.size());
    b->haveDt = true;
    if (b->planOnly) return SDG_OK;
    SDG_CUDA(cudaSetDevice(b->device));
    if (!b->built) build(b);
    else refreshArgs(b);
  } catch (const Failure& f) {
    return batchFail(b, f);
  }
  return SDG_OK;
}

int sdg_batch_set_persistence(sdg_batch* b, int32_t ctas) {
  if (!b || ctas < 0 || ctas > 64) return SDG_ERR_INVALID_ARGUMENT;
  try {
    b->persist = ctas;
    if (!b->planOnly) SDG_CUDA(cudaSetDevice(b->device));
    for (Group& g : b->groups) g.grid = persistentGrid(b, g);
    dropExec(b);
  } catch (const Failure& f) {
    return batchFail(b, f);
  }
  return SDG_OK;
}

int sdg_batch_step_async(sdg_batch* b, int32_t steps) {
  if (!b || steps < 0) return SDG_ERR_INVALID_ARGUMENT;
  try {
    if (b->planOnly) throw Failure(SDG_ERR_STATE, "the batch holds host-only instances: it can only plan");
    SDG_CUDA(cudaSetDevice(b->device));
    stepBatch(b, steps);
    if (steps > 0)
      for (sdg_handle* h : b->inst) h->gradInput = stepGradientInput(h);
  } catch (const Failure& f) {
    return batchFail(b, f);
  }
  return SDG_OK;
}

int sdg_batch_step_sequential_async(sdg_batch* b, int32_t steps) {
  if (!b || steps < 0) return SDG_ERR_INVALID_ARGUMENT;
  try {
    if (b->planOnly) throw Failure(SDG_ERR_STATE, "the batch holds host-only instances: it can only plan");
    if (!b->haveDt) throw Failure(SDG_ERR_STATE, "sdg_batch_set_delta_time before the first step");
    SDG_CUDA(cudaSetDevice(b->device));
    if (!b->built) build(b);
    for (sdg_handle* h : b->inst) {
      h->stateVersion++;
      if (steps > 0) h->gradInput = stepGradientInput(h);
    }
    for (int s = 0; s < steps; ++s)
      for (size_t i = 0; i < b->inst.size(); ++i) runRecs(b->inst[i], b->seqRecs[i], b->stream);
  } catch (const Failure& f) {
    return batchFail(b, f);
  }
  return SDG_OK;
}

int sdg_batch_synchronize(sdg_batch* b) {
  if (!b) return SDG_ERR_INVALID_ARGUMENT;
  if (b->planOnly) return SDG_OK;
  try {
    SDG_CUDA(cudaSetDevice(b->device));
    SDG_CUDA(cudaStreamSynchronize(b->stream));
    for (sdg_handle* h : b->inst) checkStatus(h);
  } catch (const Failure& f) {
    return batchFail(b, f);
  }
  return SDG_OK;
}

int sdg_batch_autotune(sdg_batch* b, int32_t flags) {
  if (!b) return SDG_ERR_INVALID_ARGUMENT;
  try {
    if (b->planOnly) throw Failure(SDG_ERR_STATE, "the batch holds host-only instances: it can only plan");
    if (!b->haveDt) throw Failure(SDG_ERR_STATE, "sdg_batch_set_delta_time before autotuning");
    SDG_CUDA(cudaSetDevice(b->device));
    SDG_CUDA(cudaStreamSynchronize(b->stream));
    // 1. tiles: tune each distinct (kernel variant) on its largest instance, share with the others
    std::map<const void*, std::pair<sdg_handle*, int>> largest;  // stage kernel -> (instance, block)
    for (sdg_handle* h : b->inst)
      for (size_t k = 0; k < h->blocks.size(); ++k) {
        const void* fn = h->blocks[k].stageV[stageSlot(h)].single;
        auto it = largest.find(fn);
        if (it == largest.end() || it->second.first->blocks[it->second.second].ne < h->blocks[k].ne)
          largest[fn] = {h, int(k)};
      }
    for (auto& kv : largest) {
      sdg_handle* h = kv.second.first;
      DevBlock& B = h->blocks[kv.second.second];
      const bool timing = h->timing;
      h->timing = false;
      const int64_t launches = h->launches;
      tuneKernel(h, B, true, flags & SDG_AUTOTUNE_RETIME);
      if (viscousPath(h)) tuneKernel(h, B, false, flags & SDG_AUTOTUNE_RETIME);
      h->timing = timing;
      h->launches = launches;
      for (sdg_handle* o : b->inst)
        for (DevBlock& C : o->blocks)
          if (C.stageV[stageSlot(o)].single == kv.first) {
            setStageTile(C, stageSlot(o), B.epb, B.threads);
            setGradTile(C, B.gepb, B.gthreads);
            dropGraph(o);
          }
    }
    build(b);
    // 2. persistence: whole batched steps, states restored afterwards
    std::vector<double*> backup(b->inst.size(), nullptr);
    for (size_t i = 0; i < b->inst.size(); ++i) {
      sdg_handle* h = b->inst[i];
      SDG_CUDA(cudaMalloc(&backup[i], h->stateCount * 8));
      SDG_CUDA(cudaMemcpyAsync(backup[i], h->state[0], h->stateCount * 8, cudaMemcpyDeviceToDevice, b->stream));
    }
    static const int kPersist[] = {0, 1, 2, 4, 8};
    float best = 1e30f;
    int pick = b->persist;
    cudaEvent_t e0, e1;
    SDG_CUDA(cudaEventCreate(&e0));
    SDG_CUDA(cudaEventCreate(&e1));
    for (int pc : kPersist) {
      b->persist = pc;
      for (Group& g : b->groups) g.grid = persistentGrid(b, g);
      capture(b);
      SDG_CUDA(cudaGraphLaunch(b->exec, b->stream));
      SDG_CUDA(cudaEventRecord(e0, b->stream));
      for (int s = 0; s < 3; ++s) SDG_CUDA(cudaGraphLaunch(b->exec, b->stream));
      SDG_CUDA(cudaEventRecord(e1, b->stream));
      SDG_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      SDG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best) { best = ms; pick = pc; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->persist = pick;
    for (Group& g : b->groups) g.grid = persistentGrid(b, g);
    dropExec(b);
    for (size_t i = 0; i < b->inst.size(); ++i) {
      sdg_handle* h = b->inst[i];
      SDG_CUDA(cudaMemcpyAsync(h->state[0], backup[i], h->stateCount * 8, cudaMemcpyDeviceToDevice, b->stream));
    }
    SDG_CUDA(cudaStreamSynchronize(b->stream));
    for (size_t i = 0; i < b->inst.size(); ++i) {
      cudaFree(backup[i]);
      traceAll(b->inst[i], 0);
      checkStatus(b->inst[i]);
    }
  } catch (const Failure& f) {
    return batchFail(b, f);
  }
  return SDG_OK;
}

int sdg_batch_get_stream(const sdg_batch* b, void** stream) {
  if (!b || !stream) return SDG_ERR_INVALID_ARGUMENT;
  *stream = b->stream;
  return SDG_OK;
}

}  // extern "C"
#pragma GCC visibility pop

// dd_batch.cu -- many single-step problems per launch of one CUDA graph.
//
// A batch holds any number of single-step problems of 1/2/4/8-bit input
// (beams with their own channel count, sample count, DM range, DM step, input
// width, zapped mask and device buffers).  Committing it records a CUDA graph
// that computes them all; results equal the plain path's bit for bit.
//
// Two forms:
//  * graph form (the default): each problem runs its own default plan (the
//    tile dd_plan_create picks without a configuration: shared partial sums
//    where they fit and save enough adds, else a direct tile).  The graph forks into a few branches, each launching
//    its share of the problems' kernels one after another (longest first,
//    shares balanced by tile cost).  The branches run concurrently, so one
//    problem's last partial wave of tiles overlaps the next problem's first.
//  * persistent form (dd_batch_set_persistent, or when some problem has no
//    default plan): one work list over all the problems' tiles, longest tiles
//    first (a tile's cost is its live rows), and a graph of [reset work
//    counter, persistent kernel].  The persistent kernel runs one CTA per
//    free slot of every SM; each CTA takes the next tile from the work
//    counter and computes it with the direct swar8 tile routine.
// A persistent kernel over the shared tile ran it 0.86-0.92x as fast per tile
// as the plain launches (a problem's fields then come from the kernel
// parameters at a runtime index, not at fixed offsets), and the persistent
// direct kernel runs at ~0.91x of the direct plain launches, so the graph
// form is the default.
//
// There is no counterpart in the reference (its test driver launches one
// kernel per configuration and beam set, src/DedispersionTest.cpp:366-399).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/dedisp_gb300.h"
#include "dd_device.cuh"

namespace dd {
void set_last_error(const char *message);
// Plan internals shared with dd_api.cu.
dd_status plan_problem(const dd_plan *plan, const void *d_input, float *d_output,
                       ProblemDesc *problem, uint64_t *rows_per_group);
dd_status plan_launch(const dd_plan *p, const ProblemDesc &P, cudaStream_t stream);
bool plan_ready(const dd_plan *p);
int plan_family(const dd_plan *p);
}

namespace {

// The batch kernel's tile configuration: the engine's default swar8 tile.
constexpr int kNW = 4, kNDT = 4, kTY = 8, kCH = 8;
constexpr int kVar = dd::kUnpackPermuteMad;
constexpr int kThreads = 32 * kTY;

struct BatchDesc {
  const dd::ProblemDesc *problems;  // sorted by tile cost, descending
  const uint32_t *tile_start;       // prefix sums of tiles, nproblems + 1
  uint32_t *counter;                // work counter (reset before each launch)
  uint32_t nproblems;
  uint32_t total_tiles;
  dd::SmemLayout layout;            // uniform over the batch
};

__global__ void __launch_bounds__(kThreads, 2) batch_kernel(const BatchDesc B) {
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ dd::ProblemDesc sP;
  __shared__ uint32_t s_tile, s_local;
  dd::init_barriers(smem, B.layout, kCH);
  uint32_t sc = 0;
  for (;;) {
    if (threadIdx.x == 0) {
      const uint32_t t = atomicAdd(B.counter, 1u);
      s_tile = t;
      if (t < B.total_tiles) {
        uint32_t lo = 0, hi = B.nproblems;  // last p with tile_start[p] <= t
        while (hi - lo > 1) {
          const uint32_t mid = (lo + hi) / 2;
          if (B.tile_start[mid] <= t) lo = mid; else hi = mid;
        }
        sP = B.problems[lo];
        s_local = t - B.tile_start[lo];
      }
    }
    __syncthreads();
    if (s_tile >= B.total_tiles) break;
    uint32_t g, dtile, ttile;
    dd::decode_tile(sP, s_local, g, dtile, ttile);
    // This problem's window and fetch size inside the batch's uniform slots.
    dd::SmemLayout L = dd::make_layout(dd::kFamilySwar8, sP.win_samples, sP.bits, kCH, kTY * kNDT);
    L.raw_stride = B.layout.raw_stride;
    L.area_words = B.layout.area_words;
    L.off_raw = B.layout.off_raw;
    L.off_copy = B.layout.off_copy;
    L.total = B.layout.total;
    const bool ok = dd::swar8_tile<kNW, kNDT, kTY, kCH, kVar>(sP, sP.groups[g], dtile, ttile,
                                                                 smem, L, sc);
    if (!ok) break;  // uniform: decided by a block-wide vote inside the tile
    __syncthreads();  // everyone is done with sP and s_tile
  }
}

// Concurrent launch chains of the graph form.
constexpr uint32_t kBranches = 4;

dd_status fail(dd_status code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  dd::set_last_error(buf);
  return code;
}

dd_status cuda_fail(cudaError_t e, const char *what) {
  (void)cudaGetLastError();
  if (e == cudaErrorMemoryAllocation)
    return fail(DD_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
  return fail(DD_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define DDB_CUDA(call, what)                           \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

}  // namespace

struct dd_batch {
  int device = 0;
  std::vector<dd_plan *> plans;         // persistent-form plans (direct tile, always built)
  std::vector<dd_plan *> shared_plans;  // each beam's default plan (NULL: none fits)
  bool shared = false;                  // committed in the graph form
  bool persistent = false;              // dd_batch_set_persistent
  std::vector<const void *> inputs;
  std::vector<float *> outputs;
  // committed state
  bool committed = false;
  dd::ProblemDesc *d_problems = nullptr;
  uint32_t *d_tile_start = nullptr;
  uint32_t *d_scratch = nullptr;  // [0] work counter, [1] status word
  BatchDesc desc{};
  // Shared-tile form: per problem its kernel arguments and branch, in
  // launch order; the branch streams and fork/join events.
  std::vector<dd::ProblemDesc> sprobs;
  std::vector<uint32_t> sbranch;
  std::vector<size_t> sorder;
  std::vector<cudaStream_t> branches;
  std::vector<cudaEvent_t> events;  // [0] fork, [1 + i] join of branch i
  uint32_t total_tiles = 0;
  size_t smem = 0;
  unsigned grid = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t capture = nullptr;
};

namespace {

void release(dd_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->capture) cudaStreamDestroy(b->capture);
  if (b->d_problems) cudaFree(b->d_problems);
  if (b->d_tile_start) cudaFree(b->d_tile_start);
  if (b->d_scratch) cudaFree(b->d_scratch);
  for (cudaStream_t s : b->branches) cudaStreamDestroy(s);
  for (cudaEvent_t e : b->events) cudaEventDestroy(e);
  b->branches.clear();
  b->events.clear();
  b->sprobs.clear();
  b->sbranch.clear();
  b->sorder.clear();
  b->exec = nullptr; b->graph = nullptr; b->capture = nullptr;
  b->d_problems = nullptr; b->d_tile_start = nullptr; b->d_scratch = nullptr;
  b->committed = false;
}

// Enqueue the batch on `s`: the forked plain launches (shared tile) or
// [counter reset, persistent kernel] (direct tile).
dd_status enqueue(dd_batch *b, cudaStream_t s) {
  if (b->shared) {
    DDB_CUDA(cudaEventRecord(b->events[0], s), "fork batch");
    for (cudaStream_t br : b->branches)
      DDB_CUDA(cudaStreamWaitEvent(br, b->events[0], 0), "fork batch");
    for (size_t k : b->sorder) {
      dd_status st = dd::plan_launch(b->shared_plans[k], b->sprobs[k], b->branches[b->sbranch[k]]);
      if (st) return st;
    }
    for (size_t i = 0; i < b->branches.size(); i++) {
      DDB_CUDA(cudaEventRecord(b->events[1 + i], b->branches[i]), "join batch");
      DDB_CUDA(cudaStreamWaitEvent(s, b->events[1 + i], 0), "join batch");
    }
    return DD_OK;
  }
  DDB_CUDA(cudaMemsetAsync(b->d_scratch, 0, sizeof(uint32_t), s), "reset work counter");
  batch_kernel<<<b->grid, kThreads, b->smem, s>>>(b->desc);
  DDB_CUDA(cudaGetLastError(), "launch batch kernel");
  return DD_OK;
}

// Shared-tile form of dd_batch_commit: each problem's arguments (status word:
// the batch's), longest-processing-time-first assignment of the problems to
// the branches by tile cost (tiles x rows per group), branch streams, events.
dd_status commit_shared(dd_batch *b) {
  const size_t n = b->plans.size();
  std::vector<uint64_t> cost(n);
  b->sprobs.resize(n);
  uint64_t total = 0;
  for (size_t i = 0; i < n; i++) {
    uint64_t rows = 0;
    dd_status st = dd::plan_problem(b->shared_plans[i], b->inputs[i], b->outputs[i],
                                    &b->sprobs[i], &rows);
    if (st) return st;
    b->sprobs[i].status = b->d_scratch + 1;
    const uint64_t tiles =
        (uint64_t)b->sprobs[i].nr_groups * b->sprobs[i].tiles_d * b->sprobs[i].tiles_t;
    cost[i] = tiles * std::max<uint64_t>(rows, 1);
    total += tiles;
  }
  if (total > 0xffffffffull) return fail(DD_ERR_UNSUPPORTED, "batch has too many tiles");
  b->total_tiles = (uint32_t)total;
  b->sorder.resize(n);
  std::iota(b->sorder.begin(), b->sorder.end(), 0);
  std::stable_sort(b->sorder.begin(), b->sorder.end(),
                   [&](size_t x, size_t y) { return cost[x] > cost[y]; });
  const uint32_t nb = (uint32_t)std::min<size_t>(kBranches, n);
  std::vector<uint64_t> load(nb, 0);
  b->sbranch.assign(n, 0);
  for (size_t k : b->sorder) {
    const uint32_t br = (uint32_t)(std::min_element(load.begin(), load.end()) - load.begin());
    b->sbranch[k] = br;
    load[br] += cost[k];
  }
  b->branches.assign(nb, nullptr);
  for (auto &br : b->branches)
    DDB_CUDA(cudaStreamCreateWithFlags(&br, cudaStreamNonBlocking), "create branch stream");
  b->events.assign(nb + 1, nullptr);
  for (auto &e : b->events)
    DDB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "create branch event");
  b->grid = nb;
  return DD_OK;
}

// Records the batch's launches as a graph (replays cost one graph launch) and
// marks it committed.
dd_status record_graph(dd_batch *b) {
  DDB_CUDA(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking), "create stream");
  DDB_CUDA(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal), "begin capture");
  dd_status st = enqueue(b, b->capture);
  cudaError_t e = cudaStreamEndCapture(b->capture, &b->graph);
  if (st) return st;
  if (e != cudaSuccess) return cuda_fail(e, "end capture");
  DDB_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0), "instantiate graph");
  b->committed = true;
  return DD_OK;
}

}  // namespace

extern "C" {

dd_status dd_batch_create(dd_batch **batch, int device) {
  if (!batch) return fail(DD_ERR_INVALID_ARGUMENT, "batch is NULL");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    (void)cudaGetLastError();
    return fail(DD_ERR_NO_DEVICE, "no CUDA device available");
  }
  if (device < 0 || device >= n) return fail(DD_ERR_INVALID_ARGUMENT, "device %d out of range", device);
  *batch = new dd_batch();
  (*batch)->device = device;
  return DD_OK;
}

dd_status dd_batch_add(dd_batch *b, const dd_observation *obs, uint32_t input_bits,
                       uint32_t padding, const float *shifts, const uint32_t *zapped,
                       const uint32_t *beam_mapping, const void *d_input, float *d_output,
                       uint32_t *index) {
  return dd_batch_add_with_kernel(b, obs, input_bits, padding, shifts, zapped, beam_mapping,
                                  d_input, d_output, -1, index);
}

dd_status dd_batch_add_with_kernel(dd_batch *b, const dd_observation *obs, uint32_t input_bits,
                                   uint32_t padding, const float *shifts, const uint32_t *zapped,
                                   const uint32_t *beam_mapping, const void *d_input,
                                   float *d_output, int kernel, uint32_t *index) {
  if (!b || !obs || !shifts || !zapped || !beam_mapping || !d_input || !d_output)
    return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (input_bits > 8) return fail(DD_ERR_UNSUPPORTED, "batches take 1/2/4/8-bit input");
  dd_conf conf{0, 1, kCH, 32, kTY, 1, 4 * kNW, kNDT, 1};
  dd_plan *p = nullptr;
  dd_status st = dd_plan_create(&p, obs, DD_SINGLE_STEP, input_bits, padding, &conf, b->device);
  if (st) return st;
  dd_layout lay;
  st = dd_get_layout(obs, DD_SINGLE_STEP, input_bits, padding, nullptr, &lay);
  if (!st) st = dd_plan_set_shifts(p, shifts, obs->nr_channels);
  if (!st) st = dd_plan_set_zapped(p, zapped, obs->nr_channels);
  if (!st) st = dd_plan_set_beam_mapping(p, beam_mapping,
                                         (size_t)obs->nr_synthesized_beams * lay.mapping_row_elems);
  if (st) {
    dd_plan_destroy(p);
    return st;
  }
  // The beam's plan for the graph form: the configuration the caller chose
  // (registry index `kernel`, e.g. a tuner's pick), or the beam's own default
  // (dd_plan_create without a configuration).
  dd_plan *q = nullptr;
  const dd_status cq =
      kernel >= 0 ? dd_plan_create_with_kernel(&q, obs, DD_SINGLE_STEP, input_bits, padding,
                                               kernel, b->device)
                  : dd_plan_create(&q, obs, DD_SINGLE_STEP, input_bits, padding, nullptr,
                                   b->device);
  if (cq == DD_OK) {
    bool good = dd_plan_set_shifts(q, shifts, obs->nr_channels) == DD_OK &&
                dd_plan_set_zapped(q, zapped, obs->nr_channels) == DD_OK &&
                dd_plan_set_beam_mapping(q, beam_mapping, (size_t)obs->nr_synthesized_beams *
                                                              lay.mapping_row_elems) == DD_OK;
    good = good && dd::plan_ready(q);
    if (!good) {
      dd_plan_destroy(q);
      q = nullptr;
    }
  }
  if (kernel >= 0 && !q) {
    dd_plan_destroy(p);
    return fail(DD_ERR_UNSUPPORTED, "configuration %d cannot run this problem", kernel);
  }
  if (b->committed) release(b);
  if (index) *index = (uint32_t)b->plans.size();
  b->plans.push_back(p);
  b->shared_plans.push_back(q);
  b->inputs.push_back(d_input);
  b->outputs.push_back(d_output);
  return DD_OK;
}

dd_status dd_batch_commit(dd_batch *b) {
  if (!b) return fail(DD_ERR_INVALID_ARGUMENT, "batch is NULL");
  if (b->plans.empty()) return fail(DD_ERR_INVALID_ARGUMENT, "batch is empty");
  release(b);
  const size_t n = b->plans.size();
  b->shared = !b->persistent &&
              std::all_of(b->shared_plans.begin(), b->shared_plans.end(),
                          [](dd_plan *q) { return q != nullptr; });
  DDB_CUDA(cudaSetDevice(b->device), "select device");
  if (b->shared) {
    DDB_CUDA(cudaMalloc(&b->d_scratch, 2 * sizeof(uint32_t)), "allocate status word");
    DDB_CUDA(cudaMemset(b->d_scratch, 0, 2 * sizeof(uint32_t)), "clear batch scratch");
    if (dd_status st = commit_shared(b)) return st;
    return record_graph(b);
  }
  std::vector<dd::ProblemDesc> probs(n);
  std::vector<uint64_t> rows(n);
  for (size_t i = 0; i < n; i++) {
    dd_status st = dd::plan_problem(b->plans[i], b->inputs[i], b->outputs[i], &probs[i], &rows[i]);
    if (st) return st;
  }
  // Uniform slots sized for the largest raw row and copy of any problem; each
  // tile fetches and builds only its own problem's window inside them.
  dd::SmemLayout L{};
  uint32_t raw_stride = 0, copy_words = 0;
  for (auto &P : probs) {
    const dd::SmemLayout l = dd::make_layout(dd::kFamilySwar8, P.win_samples, P.bits, kCH, kTY * kNDT);
    raw_stride = std::max(raw_stride, l.raw_bytes);
    copy_words = std::max(copy_words, l.copy_words);
  }
  L.raw_bytes = raw_stride;
  L.raw_stride = raw_stride;
  L.copy_words = copy_words;
  L.area_words = kCH * 4u * copy_words;
  L.off_bar = 0;
  L.off_wstart = 64;
  L.off_table = dd::round_up(L.off_wstart + 2u * dd::kNRaw * kCH * 4u, 128u);
  L.off_raw = dd::round_up(L.off_table + 2u * kCH * kTY * kNDT * 4u, 128u);
  L.off_copy = dd::round_up(L.off_raw + dd::kNRaw * kCH * L.raw_stride, 128u);
  L.total = L.off_copy + 2u * L.area_words * 4u;
  // Longest tiles first: a tile's cost is the rows its group sums.
  std::vector<size_t> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t x, size_t y) { return rows[x] > rows[y]; });
  std::vector<dd::ProblemDesc> sorted(n);
  std::vector<uint32_t> start(n + 1, 0);
  uint64_t total = 0;
  for (size_t k = 0; k < n; k++) {
    sorted[k] = probs[order[k]];
    start[k] = (uint32_t)total;
    total += (uint64_t)sorted[k].nr_groups * sorted[k].tiles_d * sorted[k].tiles_t;
  }
  if (total > 0xffffffffull - 1) return fail(DD_ERR_UNSUPPORTED, "batch has too many tiles");
  start[n] = (uint32_t)total;

  int smem_max = 0, sms = 0, per_sm = 0;
  DDB_CUDA(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device),
           "query shared memory");
  DDB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device), "query SMs");
  // The kernel's own static shared memory (the problem descriptor) comes out
  // of the same per-block budget.
  const void *kfn = reinterpret_cast<const void *>(&batch_kernel);
  const int threads = kThreads;
  cudaFuncAttributes fa{};
  DDB_CUDA(cudaFuncGetAttributes(&fa, kfn), "query kernel attributes");
  const size_t static_smem = fa.sharedSizeBytes;
  if (L.total + static_smem > (size_t)smem_max)
    return fail(DD_ERR_UNSUPPORTED, "batch window needs %u bytes of shared memory", L.total);
  DDB_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                smem_max - (int)static_smem),
           "set kernel shared memory");
  DDB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, threads, L.total),
           "occupancy");
  if (per_sm < 1) return fail(DD_ERR_UNSUPPORTED, "batch kernel does not fit on an SM");
  b->smem = L.total;
  b->grid = (unsigned)std::min<uint64_t>((uint64_t)sms * per_sm, std::max<uint64_t>(1, total));

  for (auto &P : sorted) P.status = nullptr;
  DDB_CUDA(cudaMalloc(&b->d_problems, n * sizeof(dd::ProblemDesc)), "allocate problems");
  DDB_CUDA(cudaMalloc(&b->d_tile_start, (n + 1) * sizeof(uint32_t)), "allocate tile table");
  DDB_CUDA(cudaMalloc(&b->d_scratch, 2 * sizeof(uint32_t)), "allocate work counter");
  for (auto &P : sorted) P.status = b->d_scratch + 1;
  DDB_CUDA(cudaMemset(b->d_scratch, 0, 2 * sizeof(uint32_t)), "clear batch scratch");
  DDB_CUDA(cudaMemcpy(b->d_problems, sorted.data(), n * sizeof(dd::ProblemDesc),
                      cudaMemcpyHostToDevice), "upload problems");
  DDB_CUDA(cudaMemcpy(b->d_tile_start, start.data(), (n + 1) * sizeof(uint32_t),
                      cudaMemcpyHostToDevice), "upload tile table");
  b->desc.problems = b->d_problems;
  b->desc.tile_start = b->d_tile_start;
  b->desc.counter = b->d_scratch;
  b->desc.nproblems = (uint32_t)n;
  b->desc.total_tiles = (uint32_t)total;
  b->desc.layout = L;
  b->total_tiles = (uint32_t)total;
  return record_graph(b);
}

dd_status dd_batch_run(dd_batch *b, void *stream, int use_graph) {
  if (!b) return fail(DD_ERR_INVALID_ARGUMENT, "batch is NULL");
  if (!b->committed) return fail(DD_ERR_INVALID_ARGUMENT, "batch is not committed");
  DDB_CUDA(cudaSetDevice(b->device), "select device");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (use_graph) {
    DDB_CUDA(cudaGraphLaunch(b->exec, s), "launch graph");
    return DD_OK;
  }
  return enqueue(b, s);
}

dd_status dd_batch_check(dd_batch *b, void *stream) {
  if (!b) return fail(DD_ERR_INVALID_ARGUMENT, "batch is NULL");
  if (!b->committed) return fail(DD_ERR_INVALID_ARGUMENT, "batch is not committed");
  DDB_CUDA(cudaSetDevice(b->device), "select device");
  DDB_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "synchronize stream");
  uint32_t status = 0;
  DDB_CUDA(cudaMemcpy(&status, b->d_scratch + 1, sizeof(status), cudaMemcpyDeviceToHost),
           "read status");
  if (status) {
    cudaMemset(b->d_scratch + 1, 0, sizeof(uint32_t));
    return fail(DD_ERR_TIMEOUT, "a bounded wait for a staged row ran out on the device");
  }
  return DD_OK;
}

dd_status dd_batch_info(const dd_batch *b, uint32_t *problems, uint32_t *tiles, uint32_t *grid) {
  if (!b) return fail(DD_ERR_INVALID_ARGUMENT, "batch is NULL");
  if (problems) *problems = (uint32_t)b->plans.size();
  if (tiles) *tiles = b->committed ? b->total_tiles : 0;
  if (grid) *grid = b->committed ? b->grid : 0;
  return DD_OK;
}

dd_status dd_batch_set_persistent(dd_batch *b, int enable) {
  if (!b) return fail(DD_ERR_INVALID_ARGUMENT, "batch is NULL");
  b->persistent = enable != 0;
  if (b->committed) release(b);
  return DD_OK;
}

dd_status dd_batch_shared(const dd_batch *b, int *shared) {
  if (!b || !shared) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!b->committed) return fail(DD_ERR_INVALID_ARGUMENT, "batch is not committed");
  *shared = b->shared ? 1 : 0;
  return DD_OK;
}

dd_status dd_batch_destroy(dd_batch *b) {
  if (!b) return DD_OK;
  cudaSetDevice(b->device);
  release(b);
  for (dd_plan *p : b->plans) dd_plan_destroy(p);
  for (dd_plan *q : b->shared_plans)
    if (q) dd_plan_destroy(q);
  delete b;
  return DD_OK;
}

}  // extern "C"

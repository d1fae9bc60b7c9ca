// dd_stream.cu -- one beam of a real-time dedispersion stream.
//
// Batch k of a beam brings S new samples per channel.  Dedispersing them
// needs the max-delay tail of the samples before them, so the stream keeps,
// on the device, a ring of rows [tail | S new samples] (tail = S_disp - S, or
// S1_disp - S in subband mode).  One push enqueues, as a recorded CUDA graph:
//
//   1. copy the S new samples from the stream's pinned staging buffer into
//      the ring after the tail,
//   2. dedisperse the ring (one single-step plan, or step one into a device
//      intermediate and step two from it; the intermediate is packed, two
//      coarse DMs' 16-bit sums per word, where the sums fit 16 bits),
//   3. copy the output's valid samples into the pinned output buffer,
//   4. carry the last `tail` samples of every row to the front of the ring.
//
// Output k is therefore the dedispersion of stream samples
// [k*S - tail, (k + 1)*S - tail + tail) with zeros before the first batch, and
// equals the plain path on that window bit for bit.  Device bytes are known
// before creation (dd_stream_bytes) so that a server can admit beams against
// a memory budget.  No counterpart in the reference, whose splitBatches mode
// was left unimplemented (include/Dedispersion.hpp:202; README.md:76-79).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/dedisp_gb300.h"
#include "dd_internal.h"

namespace dd {
void set_last_error(const char *message);
bool subband_packable(const dd_observation *o, const uint32_t *zapped, uint32_t bits);
bool subband_try_pack(dd_plan *one, dd_plan *two, const dd_observation *o, const uint32_t *zapped,
                      uint32_t bits, int pair_kernel);
}

namespace {

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

#define DDS_CUDA(call, what)                           \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

uint64_t pad(uint64_t v, uint64_t p) { return p == 0 ? v : (v + p - 1) / p * p; }

// Samples a byte holds (1 for >= 8 bits).
uint32_t per_byte(uint32_t bits) { return bits < 8 ? 8 / bits : 1; }
uint64_t bytes_of(uint64_t samples, uint32_t bits) {
  return bits < 8 ? samples / per_byte(bits) : samples * (bits / 8);
}

// Geometry of a stream: the observations its plans run on.
struct Geometry {
  dd_observation one;   // single step, or step one (ring input)
  dd_observation two;   // step two (subband mode)
  uint32_t tail = 0;    // carried samples
  dd_layout ring{}, mid{}, out{};
  bool packed = false;  // subband mode: packed step-one intermediate
};

dd_status geometry(const dd_observation *o, int subband, uint32_t bits, uint32_t padding,
                   const float *shifts, const float *shifts2, const uint32_t *zapped,
                   Geometry *g) {
  if (!o || !shifts || !zapped) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (subband && !shifts2) return fail(DD_ERR_INVALID_ARGUMENT, "subband streams need step-two shifts");
  const uint32_t S = o->nr_samples_per_batch;
  const uint32_t unit = per_byte(bits);
  if (S == 0 || S % unit) return fail(DD_ERR_INVALID_ARGUMENT, "samples per batch must be a positive multiple of %u", unit);
  auto max_delay = [&](const float *sh, uint32_t n, const uint32_t *z, uint32_t dms, float first,
                       float step, int relative, uint32_t cps) {
    uint32_t m = 0;
    if (dms == 0) return m;
    for (uint32_t c = 0; c < n; c++) {
      if (z && z[c]) continue;
      float s = sh[c];
      if (relative) {
        volatile float rel = sh[c] - sh[(c / cps + 1) * cps - 1];
        s = rel;
      }
      m = std::max(m, dd::host_delay(first, step, dms - 1, s));
    }
    return m;
  };
  g->one = *o;
  if (!subband) {
    uint32_t tail = max_delay(shifts, o->nr_channels, zapped, o->nr_dms, o->first_dm, o->dm_step, 0, 1);
    tail = (tail + unit - 1) / unit * unit;
    g->tail = tail;
    g->one.nr_samples_per_dispersed_batch = S + tail;
    dd_status st = dd_get_layout(&g->one, DD_SINGLE_STEP, bits, padding, nullptr, &g->ring);
    if (st) return st;
    g->out = g->ring;
  } else {
    if (o->nr_subbands == 0 || o->nr_channels % o->nr_subbands)
      return fail(DD_ERR_INVALID_ARGUMENT, "channels must split evenly into subbands");
    const uint32_t cps = o->nr_channels / o->nr_subbands;
    const uint32_t d2 = max_delay(shifts2, o->nr_subbands, nullptr, o->nr_dms, o->first_dm, o->dm_step, 0, 1);
    const uint32_t S1 = S + d2;
    uint32_t d1 = max_delay(shifts, o->nr_channels, zapped, o->nr_dms_subbanding,
                            o->first_dm_subbanding, o->dm_step_subbanding, 1, cps);
    uint32_t tail = (S1 - S) + d1;
    tail = (tail + unit - 1) / unit * unit;
    g->tail = tail;
    g->one.nr_samples_per_batch_subbanding = S1;
    g->one.nr_samples_per_dispersed_batch_subbanding = S + tail;
    g->two = g->one;
    g->two.nr_beams = 1;
    g->two.nr_synthesized_beams = 1;
    dd_status st = dd_get_layout(&g->one, DD_STEP_ONE, bits, padding, nullptr, &g->ring);
    if (!st) st = dd_get_layout(&g->two, DD_STEP_TWO, 32, padding, nullptr, &g->out);
    if (st) return st;
    g->mid = g->ring;
    g->packed = dd::subband_packable(&g->one, zapped, bits);
  }
  if (g->tail > S) return fail(DD_ERR_UNSUPPORTED, "max delay %u exceeds the batch of %u samples", g->tail, S);
  if (o->nr_beams != 1 || o->nr_synthesized_beams != 1)
    return fail(DD_ERR_UNSUPPORTED, "a stream carries one beam");
  return DD_OK;
}

}  // namespace

struct dd_stream {
  int device = 0;
  int subband = 0;
  uint32_t bits = 8, padding = 0;
  Geometry g;
  dd_plan *plan1 = nullptr, *plan2 = nullptr;
  uint8_t *d_ring = nullptr;
  float *d_mid = nullptr, *d_out = nullptr;
  // Pinned staging input and output, one pair per buffer; push k uses pair
  // k % nbuf (dd_stream_set_double_buffer: nbuf = 2).
  uint8_t *h_in[2] = {nullptr, nullptr};
  float *h_out[2] = {nullptr, nullptr};
  int nbuf = 1, next = 0;
  uint64_t device_bytes = 0;
  uint64_t in_row_bytes = 0;  // staging row: S samples
  uint32_t out_rows = 0;
  cudaStream_t capture = nullptr;
  cudaGraph_t graph[2] = {nullptr, nullptr};
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  // Time-major input (dd_stream_set_time_major): the staged block [S][C] is
  // copied to d_block and transposed into the ring.
  bool time_major = false;
  int reverse = 0;
  uint8_t *d_block = nullptr;
};

namespace {

void release(dd_stream *s) {
  for (int b = 0; b < 2; b++) {
    if (s->exec[b]) cudaGraphExecDestroy(s->exec[b]);
    if (s->graph[b]) cudaGraphDestroy(s->graph[b]);
  }
  if (s->capture) cudaStreamDestroy(s->capture);
  if (s->plan1) dd_plan_destroy(s->plan1);
  if (s->plan2) dd_plan_destroy(s->plan2);
  if (s->d_ring) cudaFree(s->d_ring);
  if (s->d_mid) cudaFree(s->d_mid);
  if (s->d_out) cudaFree(s->d_out);
  for (int b = 0; b < 2; b++) {
    if (s->h_in[b]) cudaFreeHost(s->h_in[b]);
    if (s->h_out[b]) cudaFreeHost(s->h_out[b]);
  }
  if (s->d_block) cudaFree(s->d_block);
}

// Bytes of the step-one intermediate: the float rows, or half as many packed
// rows (pairs of coarse DMs) when the sums fit 16 bits.
uint64_t mid_bytes(const Geometry &g) {
  const uint64_t D1 = g.one.nr_dms_subbanding;
  if (!g.packed || D1 == 0) return g.ring.output_bytes;
  return g.ring.output_bytes / D1 * ((D1 + 1) / 2);
}

uint64_t total_bytes(const Geometry &g, int subband) {
  uint64_t b = g.ring.input_bytes + g.out.output_bytes;
  if (subband) b += mid_bytes(g);  // step-one intermediate
  return b;
}

dd_status enqueue(dd_stream *s, cudaStream_t st, int buf);

// (Re-)records the push as a graph, one per staging buffer.
dd_status record(dd_stream *s) {
  for (int b = 0; b < 2; b++) {
    if (s->exec[b]) cudaGraphExecDestroy(s->exec[b]);
    if (s->graph[b]) cudaGraphDestroy(s->graph[b]);
    s->exec[b] = nullptr;
    s->graph[b] = nullptr;
  }
  if (!s->capture) DDS_CUDA(cudaStreamCreateWithFlags(&s->capture, cudaStreamNonBlocking), "create stream");
  for (int b = 0; b < s->nbuf; b++) {
    DDS_CUDA(cudaStreamBeginCapture(s->capture, cudaStreamCaptureModeThreadLocal), "begin capture");
    dd_status st = enqueue(s, s->capture, b);
    cudaError_t e = cudaStreamEndCapture(s->capture, &s->graph[b]);
    if (st) return st;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&s->exec[b], s->graph[b], 0);
    // Upload now, so that the first push of each buffer does not pay for it
    // inside a served batch's latency.
    if (e == cudaSuccess) e = cudaGraphUpload(s->exec[b], s->capture);
    if (e != cudaSuccess) return cuda_fail(e, "record stream graph");
  }
  DDS_CUDA(cudaStreamSynchronize(s->capture), "upload stream graphs");
  return DD_OK;
}

dd_status enqueue(dd_stream *s, cudaStream_t st, int buf) {
  const Geometry &g = s->g;
  const uint32_t C = g.one.nr_channels, S = g.one.nr_samples_per_batch;
  const uint64_t tail_b = bytes_of(g.tail, s->bits), new_b = bytes_of(S, s->bits);
  // 1. new samples after the tail (channel rows, or a time-major block
  //    transposed into the rows on the device)
  if (s->time_major) {
    DDS_CUDA(cudaMemcpyAsync(s->d_block, s->h_in[buf], (size_t)S * C, cudaMemcpyHostToDevice, st),
             "copy batch");
    dd_status r = dd_transpose_time_major(s->d_block, S, C, s->reverse, s->d_ring,
                                          g.ring.input_row_bytes, g.tail, st);
    if (r) return r;
  } else {
    DDS_CUDA(cudaMemcpy2DAsync(s->d_ring + tail_b, g.ring.input_row_bytes, s->h_in[buf],
                               s->in_row_bytes, new_b, C, cudaMemcpyHostToDevice, st),
             "copy batch to ring");
  }
  // 2. dedisperse
  dd_status r = dd_plan_run(s->plan1, s->d_ring, s->subband ? s->d_mid : s->d_out, st);
  if (!r && s->subband) r = dd_plan_run(s->plan2, s->d_mid, s->d_out, st);
  if (r) return r;
  // 3. valid output samples to the pinned host rows
  DDS_CUDA(cudaMemcpy2DAsync(s->h_out[buf], (size_t)S * 4, s->d_out, g.out.output_row_elems * 4,
                             (size_t)S * 4, s->out_rows, cudaMemcpyDeviceToHost, st),
           "copy output");
  // 4. carry the tail to the front (source and destination do not overlap: S >= tail)
  if (tail_b)
    DDS_CUDA(cudaMemcpy2DAsync(s->d_ring, g.ring.input_row_bytes, s->d_ring + new_b,
                               g.ring.input_row_bytes, tail_b, C, cudaMemcpyDeviceToDevice, st),
             "carry tail");
  return DD_OK;
}

}  // namespace

extern "C" {

dd_status dd_stream_bytes(const dd_observation *obs, int subband, uint32_t input_bits,
                          uint32_t padding, const float *shifts, const float *shifts_step_two,
                          const uint32_t *zapped, uint64_t *device_bytes, uint32_t *tail) {
  if (!device_bytes) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  Geometry g;
  dd_status st = geometry(obs, subband, input_bits, padding, shifts, shifts_step_two, zapped, &g);
  if (st) return st;
  *device_bytes = total_bytes(g, subband);
  if (tail) *tail = g.tail;
  return DD_OK;
}

dd_status dd_stream_create(dd_stream **out, const dd_observation *obs, int subband,
                           uint32_t input_bits, uint32_t padding, const float *shifts,
                           const float *shifts_step_two, const uint32_t *zapped, int device) {
  if (!out) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = nullptr;
  if (input_bits != 1 && input_bits != 2 && input_bits != 4 && input_bits != 8 &&
      input_bits != 16 && input_bits != 32)
    return fail(DD_ERR_UNSUPPORTED, "input_bits %u not supported", input_bits);
  dd_stream *s = new dd_stream();
  s->device = device;
  s->subband = subband ? 1 : 0;
  s->bits = input_bits;
  s->padding = padding;
  dd_status st = geometry(obs, s->subband, input_bits, padding, shifts, shifts_step_two, zapped, &s->g);
  auto bail = [&](dd_status code) {
    release(s);
    delete s;
    return code;
  };
  if (st) return bail(st);
  if (cudaSetDevice(device) != cudaSuccess) {
    (void)cudaGetLastError();
    return bail(fail(DD_ERR_NO_DEVICE, "cannot select device %d", device));
  }
  const Geometry &g = s->g;
  const uint32_t C = g.one.nr_channels, S = g.one.nr_samples_per_batch;
  // plans
  st = dd_plan_create(&s->plan1, &g.one, s->subband ? DD_STEP_ONE : DD_SINGLE_STEP, input_bits,
                      padding, nullptr, device);
  if (!st) st = dd_plan_set_shifts(s->plan1, shifts, C);
  if (!st) st = dd_plan_set_zapped(s->plan1, zapped, C);
  if (!st && !s->subband) {
    std::vector<uint32_t> map(g.ring.mapping_row_elems, 0);
    st = dd_plan_set_beam_mapping(s->plan1, map.data(), map.size());
  }
  if (!st && s->subband) {
    st = dd_plan_create(&s->plan2, &g.two, DD_STEP_TWO, 32, padding, nullptr, device);
    std::vector<uint32_t> map(g.out.mapping_row_elems, 0);
    if (!st) st = dd_plan_set_shifts(s->plan2, shifts_step_two, g.two.nr_subbands);
    if (!st) st = dd_plan_set_beam_mapping(s->plan2, map.data(), map.size());
    // The packed intermediate where the step-one sums fit 16 bits.
    if (!st) s->g.packed = dd::subband_try_pack(s->plan1, s->plan2, &g.one, zapped, input_bits, 0);
  }
  // Build the plans' tables now (they are built on first use), so that the
  // push recorded as a graph below launches only kernels.
  uint64_t adds = 0;
  if (!st) st = dd_plan_adds(s->plan1, &adds);
  if (!st && s->subband) st = dd_plan_adds(s->plan2, &adds);
  if (st) return bail(st);
  // buffers
  s->in_row_bytes = bytes_of(S, input_bits);
  s->out_rows = (uint32_t)(g.out.output_bytes / 4 / g.out.output_row_elems);
  cudaError_t e = cudaMalloc(&s->d_ring, g.ring.input_bytes);
  if (e == cudaSuccess) e = cudaMemset(s->d_ring, 0, g.ring.input_bytes);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_out, g.out.output_bytes);
  if (e == cudaSuccess && s->subband) e = cudaMalloc(&s->d_mid, mid_bytes(g));
  if (e == cudaSuccess) e = cudaHostAlloc(&s->h_in[0], s->in_row_bytes * C, cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaMemset(s->d_out, 0, g.out.output_bytes);
  if (e == cudaSuccess)
    e = cudaHostAlloc(reinterpret_cast<void **>(&s->h_out[0]), (size_t)S * 4 * s->out_rows,
                      cudaHostAllocDefault);
  if (e != cudaSuccess) return bail(cuda_fail(e, "allocate stream buffers"));
  std::memset(s->h_in[0], 0, s->in_row_bytes * C);
  s->device_bytes = total_bytes(g, s->subband);
  st = record(s);
  if (st) return bail(st);
  *out = s;
  return DD_OK;
}

dd_status dd_stream_set_time_major(dd_stream *s, int reverse) {
  if (!s) return fail(DD_ERR_INVALID_ARGUMENT, "stream is NULL");
  if (s->bits != 8) return fail(DD_ERR_UNSUPPORTED, "time-major input takes 8-bit samples");
  DDS_CUDA(cudaSetDevice(s->device), "select device");
  const uint64_t bytes = (uint64_t)s->g.one.nr_samples_per_batch * s->g.one.nr_channels;
  if (!s->d_block) DDS_CUDA(cudaMalloc(&s->d_block, std::max<uint64_t>(bytes, 16)), "allocate block");
  s->time_major = true;
  s->reverse = reverse ? 1 : 0;
  s->device_bytes = total_bytes(s->g, s->subband) + bytes;
  return record(s);
}

dd_status dd_stream_buffers(dd_stream *s, void **h_input, float **h_output, float **d_output) {
  if (!s) return fail(DD_ERR_INVALID_ARGUMENT, "stream is NULL");
  if (h_input) *h_input = s->h_in[s->next];
  if (h_output) *h_output = s->h_out[s->next];
  if (d_output) *d_output = s->d_out;
  return DD_OK;
}

dd_status dd_stream_info(const dd_stream *s, uint32_t *tail, uint64_t *device_bytes,
                         uint64_t *input_row_bytes, uint32_t *output_rows) {
  if (!s) return fail(DD_ERR_INVALID_ARGUMENT, "stream is NULL");
  if (tail) *tail = s->g.tail;
  if (device_bytes) *device_bytes = s->device_bytes;
  if (input_row_bytes) *input_row_bytes = s->in_row_bytes;
  if (output_rows) *output_rows = s->out_rows;
  return DD_OK;
}

dd_status dd_stream_push(dd_stream *s, void *stream) {
  if (!s) return fail(DD_ERR_INVALID_ARGUMENT, "stream is NULL");
  DDS_CUDA(cudaSetDevice(s->device), "select device");
  DDS_CUDA(cudaGraphLaunch(s->exec[s->next], static_cast<cudaStream_t>(stream)),
           "launch stream graph");
  s->next = (s->next + 1) % s->nbuf;
  return DD_OK;
}

dd_status dd_stream_set_double_buffer(dd_stream *s, int enable) {
  if (!s) return fail(DD_ERR_INVALID_ARGUMENT, "stream is NULL");
  DDS_CUDA(cudaSetDevice(s->device), "select device");
  const uint32_t C = s->g.one.nr_channels, S = s->g.one.nr_samples_per_batch;
  if (enable && !s->h_in[1]) {
    DDS_CUDA(cudaHostAlloc(&s->h_in[1], s->in_row_bytes * C, cudaHostAllocDefault),
             "allocate staging");
    std::memset(s->h_in[1], 0, s->in_row_bytes * C);
    DDS_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&s->h_out[1]), (size_t)S * 4 * s->out_rows,
                           cudaHostAllocDefault),
             "allocate output");
  }
  s->nbuf = enable ? 2 : 1;
  s->next = 0;
  return record(s);
}

dd_status dd_stream_buffer(dd_stream *s, int index, void **h_input, float **h_output) {
  if (!s) return fail(DD_ERR_INVALID_ARGUMENT, "stream is NULL");
  if (index < 0 || index >= s->nbuf)
    return fail(DD_ERR_INVALID_ARGUMENT, "buffer %d of %d", index, s->nbuf);
  if (h_input) *h_input = s->h_in[index];
  if (h_output) *h_output = s->h_out[index];
  return DD_OK;
}

dd_status dd_stream_next_buffer(const dd_stream *s, int *index) {
  if (!s || !index) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  *index = s->next;
  return DD_OK;
}

dd_status dd_stream_destroy(dd_stream *s) {
  if (!s) return DD_OK;
  cudaSetDevice(s->device);
  release(s);
  delete s;
  return DD_OK;
}

}  // extern "C"

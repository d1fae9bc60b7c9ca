/*
 * dd_oracle.c -- CPU oracle for the dedispersion hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this file: it is built into its own shared object and used by the
 * tests, by the smoke check and by bench.py's CPU baseline, always as the
 * checker and never as the thing measured for the GPU path.
 *
 * It restates, loop for loop and in the same float expression order, the
 * reference's serial CPU code of TRASAL/Dedispersion:
 *   ddo_get_shifts            src/Shifts.cpp:20-30
 *   ddo_get_shifts_step_two   src/Shifts.cpp:32-42
 *   ddo_dedispersion          include/Dedispersion.hpp:70-109
 *   ddo_step_one              include/Dedispersion.hpp:111-153
 *   ddo_step_two              include/Dedispersion.hpp:155-176
 * Accumulation is in float (the reference's intermediate type L = float,
 * include/configuration.hpp:13), so float results match the reference bit
 * for bit.  ddo_dedispersion_f64 is the same loop accumulated in double, the
 * FP64 oracle for float32 input.
 *
 * Where the reference is broken or undefined the restatement follows its
 * evident intent, and says so at the line:
 *   - sub-byte rows of beam > 0: the reference adds the raw beamMapping value
 *     to the byte index (include/Dedispersion.hpp:97); here the beam's row
 *     block is beamMapping * C * rowBytes, as for >= 8-bit input.
 *   - sub-byte row length: the reference floors S_disp / (8 / bits)
 *     (include/Dedispersion.hpp:97); here it is rounded up.
 *   - step-one output pitch: the reference divides S1 by (8 / bits), which
 *     is a division by zero above 8 bits (include/Dedispersion.hpp:148); here
 *     the pitch is pad(S1, padding / sizeof(float)) for every input type.
 * All three agree with the reference whenever the reference is defined and
 * correct (8-bit input; sub-byte input with one beam and S_disp a multiple
 * of 8 / bits).
 *
 * Build with -std=c11 -ffp-contract=off (ISO mode, no FMA contraction), as
 * the reference is built with -std=c++14 (CMakeLists.txt:5).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/dedisp_gb300.h"

#if defined(__FP_FAST_FMAF) && !defined(DDO_ALLOW_FMA)
/* Only informative: -ffp-contract=off is what matters for a + b * c. */
#endif

/* isa::utils::pad: round up to a multiple of padding; padding 0 = none. */
static uint64_t ddo_pad(uint64_t value, uint64_t padding) {
  if (padding == 0) return value;
  return ((value + padding - 1) / padding) * padding;
}

/* AstroData::Observation::getMaxFreq: frequency of the highest channel. */
static float ddo_max_freq(const dd_observation *o) {
  return o->min_freq + ((o->nr_channels - 1) * o->channel_bandwidth);
}

/* Subband frequencies.  AstroData is not part of the reference tree; the
 * subband frequency of subband s is taken as the frequency of its highest
 * channel, the same channel step one dedisperses each subband to
 * (include/Dedispersion.hpp:124), so that step one + step two delays add up
 * to the single-step delay. */
static float ddo_subband_bandwidth(const dd_observation *o) {
  return (o->nr_channels / o->nr_subbands) * o->channel_bandwidth;
}
static float ddo_subband_min_freq(const dd_observation *o) {
  return o->min_freq +
         (((o->nr_channels / o->nr_subbands) - 1) * o->channel_bandwidth);
}
static float ddo_subband_max_freq(const dd_observation *o) {
  return ddo_subband_min_freq(o) +
         ((o->nr_subbands - 1) * ddo_subband_bandwidth(o));
}

float ddo_max_freq_c(const dd_observation *o) { return ddo_max_freq(o); }
float ddo_subband_min_freq_c(const dd_observation *o) {
  return ddo_subband_min_freq(o);
}
float ddo_subband_max_freq_c(const dd_observation *o) {
  return ddo_subband_max_freq(o);
}
float ddo_subband_bandwidth_c(const dd_observation *o) {
  return ddo_subband_bandwidth(o);
}

/* src/Shifts.cpp:20-30 */
int ddo_get_shifts(const dd_observation *o, uint32_t padding, float *shifts,
                   size_t capacity) {
  size_t n = (size_t)ddo_pad(o->nr_channels, padding / sizeof(float));
  if (o->nr_channels == 0 || capacity < n) return -1;
  float inverseHighFreq = 1.0f / powf(ddo_max_freq(o), 2.0f);
  float timeUnit = o->nr_samples_per_batch * o->sampling_time;
  memset(shifts, 0, n * sizeof(float));
  for (uint32_t channel = 0; channel < o->nr_channels - 1; channel++) {
    float inverseFreq =
        1.0f / powf(o->min_freq + (channel * o->channel_bandwidth), 2.0f);
    shifts[channel] = (4148.808f * (inverseFreq - inverseHighFreq) *
                       (o->nr_samples_per_batch / o->downsampling)) /
                      timeUnit;
  }
  shifts[o->nr_channels - 1] = 0;
  return 0;
}

/* src/Shifts.cpp:32-42 */
int ddo_get_shifts_step_two(const dd_observation *o, uint32_t padding,
                            float *shifts, size_t capacity) {
  size_t n = (size_t)ddo_pad(o->nr_subbands, padding / sizeof(float));
  if (o->nr_subbands == 0 || capacity < n) return -1;
  float inverseHighFreq = 1.0f / powf(ddo_subband_max_freq(o), 2.0f);
  float timeUnit = o->nr_samples_per_batch * o->sampling_time;
  memset(shifts, 0, n * sizeof(float));
  for (uint32_t subband = 0; subband < o->nr_subbands - 1; subband++) {
    float inverseFreq = 1.0f / powf(ddo_subband_min_freq(o) +
                                        (subband * ddo_subband_bandwidth(o)),
                                    2.0f);
    shifts[subband] = (4148.808f * (inverseFreq - inverseHighFreq) *
                       (o->nr_samples_per_batch / o->downsampling)) /
                      timeUnit;
  }
  shifts[o->nr_subbands - 1] = 0;
  return 0;
}

/* Bytes per stored sample element for an input type. */
static uint32_t ddo_elem_bytes(uint32_t bits) {
  return bits <= 8 ? 1u : bits / 8u;
}

/* Bytes between channel rows of `samples` samples. */
uint64_t ddo_row_bytes(uint32_t samples, uint32_t bits, uint32_t padding) {
  if (bits < 8) {
    uint32_t per_byte = 8 / bits;
    uint64_t bytes = (samples + per_byte - 1) / per_byte; /* rounded up */
    return ddo_pad(bytes, padding);
  }
  uint32_t eb = ddo_elem_bytes(bits);
  return ddo_pad(samples, padding / eb) * eb;
}

/* Reads sample `k` of a row as float, the way the reference converts
 * `static_cast<L>(input[...])` (>= 8 bits) or assembles the sub-byte value
 * bit by bit, zero-extended (include/Dedispersion.hpp:92-103). */
static inline float ddo_sample(const uint8_t *row, uint64_t k, uint32_t bits) {
  switch (bits) {
    case 8: return (float)row[k];
    case 16: return (float)((const uint16_t *)row)[k];
    case 32: return ((const float *)row)[k];
    default: {
      uint32_t per_byte = 8 / bits;
      uint64_t byte = k / per_byte;
      uint32_t firstBit = (uint32_t)(k % per_byte) * bits;
      uint32_t value = (row[byte] >> firstBit) & ((1u << bits) - 1u);
      return (float)value;
    }
  }
}

static inline double ddo_sample_f64(const uint8_t *row, uint64_t k,
                                    uint32_t bits) {
  if (bits == 32) return (double)((const float *)row)[k];
  return (double)ddo_sample(row, k, bits);
}

/* ---------------------------------------------------------------------- */
/* Work split across threads: item = (group, dm) pairs.                     */

typedef struct ddo_job {
  const dd_observation *o;
  const uint32_t *zapped;
  const uint32_t *mapping;
  const uint8_t *in;
  void *out;
  const float *shifts;
  uint32_t padding, bits;
  uint32_t dm_begin, dm_end; /* dm sub-range of single step */
  int f64;
  uint64_t item_begin, item_end;
  int mode;
} ddo_job;

/* include/Dedispersion.hpp:70-109, one (sBeam, dm) item. */
static void ddo_single_item(const ddo_job *j, uint32_t sBeam, uint32_t dm) {
  const dd_observation *o = j->o;
  uint32_t C = o->nr_channels;
  uint64_t rowBytes =
      ddo_row_bytes(o->nr_samples_per_dispersed_batch, j->bits, j->padding);
  uint64_t mapPitch = ddo_pad(C, j->padding / sizeof(uint32_t));
  uint64_t outPitch = ddo_pad(o->nr_samples_per_batch / o->downsampling,
                              j->padding / sizeof(float));
  uint32_t S = o->nr_samples_per_batch / o->downsampling;
  for (uint32_t sample = 0; sample < S; sample++) {
    float acc = 0.0f;
    double acc64 = 0.0;
    for (uint32_t channel = 0; channel < C; channel++) {
      unsigned int shift = (unsigned int)((o->first_dm + (dm * o->dm_step)) *
                                          j->shifts[channel]);
      if (j->zapped[channel] != 0) continue;
      uint64_t beam = j->mapping[(sBeam * mapPitch) + channel];
      const uint8_t *row = j->in + (beam * C + channel) * rowBytes;
      if (j->f64)
        acc64 += ddo_sample_f64(row, (uint64_t)sample + shift, j->bits);
      else
        acc += ddo_sample(row, (uint64_t)sample + shift, j->bits);
    }
    uint64_t idx = ((uint64_t)sBeam * o->nr_dms * outPitch) +
                   ((uint64_t)dm * outPitch) + sample;
    if (j->f64)
      ((double *)j->out)[idx] = acc64;
    else
      ((float *)j->out)[idx] = acc;
  }
}

/* include/Dedispersion.hpp:111-153, one (beam, dm, subband) item. */
static void ddo_step_one_item(const ddo_job *j, uint32_t beam, uint32_t dm,
                              uint32_t subband) {
  const dd_observation *o = j->o;
  uint32_t C = o->nr_channels;
  uint32_t cps = C / o->nr_subbands;
  uint32_t S1 = o->nr_samples_per_batch_subbanding / o->downsampling;
  uint64_t rowBytes = ddo_row_bytes(
      o->nr_samples_per_dispersed_batch_subbanding, j->bits, j->padding);
  uint64_t outPitch = ddo_pad(S1, j->padding / sizeof(float));
  for (uint32_t sample = 0; sample < S1; sample++) {
    float acc = 0.0f;
    for (uint32_t channel = subband * cps; channel < (subband + 1) * cps;
         channel++) {
      unsigned int shift = (unsigned int)(
          (o->first_dm_subbanding + (dm * o->dm_step_subbanding)) *
          (j->shifts[channel] - j->shifts[((subband + 1) * cps) - 1]));
      if (j->zapped[channel] != 0) continue;
      const uint8_t *row = j->in + ((uint64_t)beam * C + channel) * rowBytes;
      acc += ddo_sample(row, (uint64_t)sample + shift, j->bits);
    }
    uint64_t idx = ((uint64_t)beam * o->nr_dms_subbanding * o->nr_subbands *
                    outPitch) +
                   ((uint64_t)dm * o->nr_subbands * outPitch) +
                   ((uint64_t)subband * outPitch) + sample;
    ((float *)j->out)[idx] = acc;
  }
}

/* include/Dedispersion.hpp:155-176, one (sBeam, firstStepDM, dm) item. */
static void ddo_step_two_item(const ddo_job *j, uint32_t sBeam,
                              uint32_t firstStepDM, uint32_t dm) {
  const dd_observation *o = j->o;
  uint32_t SB = o->nr_subbands;
  uint32_t D1 = o->nr_dms_subbanding;
  uint32_t S = o->nr_samples_per_batch / o->downsampling;
  uint64_t inPitch =
      ddo_pad(o->nr_samples_per_batch_subbanding / o->downsampling,
              j->padding / sizeof(float));
  uint64_t outPitch = ddo_pad(S, j->padding / sizeof(float));
  uint64_t mapPitch = ddo_pad(SB, j->padding / sizeof(uint32_t));
  const float *in = (const float *)j->in;
  for (uint32_t sample = 0; sample < S; sample++) {
    float acc = 0.0f;
    for (uint32_t channel = 0; channel < SB; channel++) {
      unsigned int shift = (unsigned int)((o->first_dm + (dm * o->dm_step)) *
                                          j->shifts[channel]);
      uint64_t beam = j->mapping[(sBeam * mapPitch) + channel];
      acc += in[(beam * D1 * SB * inPitch) + ((uint64_t)firstStepDM * SB *
                                              inPitch) +
                (channel * inPitch) + ((uint64_t)sample + shift)];
    }
    uint64_t idx = ((uint64_t)sBeam * (D1 * o->nr_dms) * outPitch) +
                   ((((uint64_t)firstStepDM * o->nr_dms) + dm) * outPitch) +
                   sample;
    ((float *)j->out)[idx] = acc;
  }
}

static void *ddo_worker(void *arg) {
  const ddo_job *j = (const ddo_job *)arg;
  const dd_observation *o = j->o;
  for (uint64_t it = j->item_begin; it < j->item_end; it++) {
    if (j->mode == DD_SINGLE_STEP) {
      uint32_t nd = j->dm_end - j->dm_begin;
      ddo_single_item(j, (uint32_t)(it / nd), j->dm_begin + (uint32_t)(it % nd));
    } else if (j->mode == DD_STEP_ONE) {
      uint64_t per_beam = (uint64_t)o->nr_dms_subbanding * o->nr_subbands;
      uint32_t beam = (uint32_t)(it / per_beam);
      uint64_t r = it % per_beam;
      ddo_step_one_item(j, beam, (uint32_t)(r / o->nr_subbands),
                        (uint32_t)(r % o->nr_subbands));
    } else {
      uint64_t per_beam = (uint64_t)o->nr_dms_subbanding * o->nr_dms;
      uint32_t sBeam = (uint32_t)(it / per_beam);
      uint64_t r = it % per_beam;
      ddo_step_two_item(j, sBeam, (uint32_t)(r / o->nr_dms),
                        (uint32_t)(r % o->nr_dms));
    }
  }
  return NULL;
}

static int ddo_run(ddo_job *tmpl, uint64_t items, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if ((uint64_t)nthreads > items) nthreads = (int)(items ? items : 1);
  pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
  ddo_job *jobs = (ddo_job *)calloc((size_t)nthreads, sizeof(ddo_job));
  if (!th || !jobs) {
    free(th);
    free(jobs);
    return -1;
  }
  for (int t = 0; t < nthreads; t++) {
    jobs[t] = *tmpl;
    jobs[t].item_begin = items * (uint64_t)t / (uint64_t)nthreads;
    jobs[t].item_end = items * (uint64_t)(t + 1) / (uint64_t)nthreads;
  }
  for (int t = 1; t < nthreads; t++)
    pthread_create(&th[t], NULL, ddo_worker, &jobs[t]);
  ddo_worker(&jobs[0]);
  for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
  free(th);
  free(jobs);
  return 0;
}

static int ddo_bits_ok(uint32_t bits) {
  return bits == 1 || bits == 2 || bits == 4 || bits == 8 || bits == 16 ||
         bits == 32;
}

/* Single step over DMs [dm_begin, dm_end) (rows outside are not written);
 * dm_end = 0 means all DMs. */
int ddo_dedispersion(const dd_observation *o, const uint32_t *zapped,
                     const uint32_t *mapping, const void *input, float *output,
                     const float *shifts, uint32_t padding, uint32_t bits,
                     uint32_t dm_begin, uint32_t dm_end, int nthreads) {
  if (!ddo_bits_ok(bits)) return -1;
  if (dm_end == 0) dm_end = o->nr_dms;
  if (dm_begin >= dm_end) return 0;
  ddo_job j;
  memset(&j, 0, sizeof(j));
  j.o = o; j.zapped = zapped; j.mapping = mapping; j.in = (const uint8_t *)input;
  j.out = output; j.shifts = shifts; j.padding = padding; j.bits = bits;
  j.dm_begin = dm_begin; j.dm_end = dm_end; j.mode = DD_SINGLE_STEP;
  return ddo_run(&j, (uint64_t)o->nr_synthesized_beams * (dm_end - dm_begin),
                 nthreads);
}

/* Same, accumulated in double: the FP64 oracle for float32 input. */
int ddo_dedispersion_f64(const dd_observation *o, const uint32_t *zapped,
                         const uint32_t *mapping, const void *input,
                         double *output, const float *shifts, uint32_t padding,
                         uint32_t bits, int nthreads) {
  if (!ddo_bits_ok(bits)) return -1;
  ddo_job j;
  memset(&j, 0, sizeof(j));
  j.o = o; j.zapped = zapped; j.mapping = mapping; j.in = (const uint8_t *)input;
  j.out = output; j.shifts = shifts; j.padding = padding; j.bits = bits;
  j.dm_begin = 0; j.dm_end = o->nr_dms; j.mode = DD_SINGLE_STEP; j.f64 = 1;
  return ddo_run(&j, (uint64_t)o->nr_synthesized_beams * o->nr_dms, nthreads);
}

int ddo_step_one(const dd_observation *o, const uint32_t *zapped,
                 const void *input, float *output, const float *shifts,
                 uint32_t padding, uint32_t bits, int nthreads) {
  if (!ddo_bits_ok(bits) || o->nr_subbands == 0) return -1;
  ddo_job j;
  memset(&j, 0, sizeof(j));
  j.o = o; j.zapped = zapped; j.in = (const uint8_t *)input; j.out = output;
  j.shifts = shifts; j.padding = padding; j.bits = bits; j.mode = DD_STEP_ONE;
  return ddo_run(&j,
                 (uint64_t)o->nr_beams * o->nr_dms_subbanding * o->nr_subbands,
                 nthreads);
}

int ddo_step_two(const dd_observation *o, const uint32_t *mapping,
                 const float *input, float *output, const float *shifts,
                 uint32_t padding, int nthreads) {
  if (o->nr_subbands == 0) return -1;
  ddo_job j;
  memset(&j, 0, sizeof(j));
  j.o = o; j.mapping = mapping; j.in = (const uint8_t *)input; j.out = output;
  j.shifts = shifts; j.padding = padding; j.bits = 32; j.mode = DD_STEP_TWO;
  return ddo_run(&j,
                 (uint64_t)o->nr_synthesized_beams * o->nr_dms_subbanding *
                     o->nr_dms,
                 nthreads);
}

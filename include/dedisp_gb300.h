/*
 * dedisp_gb300.h -- C ABI of the GB300 incoherent dedispersion engine.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, never
 * throws, and returns a dd_status (0 = success, negative = error).  The text
 * of the most recent error on the calling thread is returned by
 * dd_last_error().  There is no CPU fallback: without a CUDA device every
 * compute entry point returns DD_ERR_NO_DEVICE.
 *
 * The algorithm is the direct-sum (brute force) dedispersion of
 * TRASAL/Dedispersion:
 *
 *   out[g][dm][t] = sum over live channels c of g of
 *                   in[row(g, c)][t + (uint)((firstDM + dm * dmStep) * shift[c])]
 *
 * in single-step form (include/Dedispersion.hpp:70-109 of the reference) and
 * in two-step subband form (include/Dedispersion.hpp:111-176).  Data layouts
 * are the reference's: rows padded to `padding` bytes (isa::utils::pad), the
 * output [synthesized beam][DM][padded samples] in float32.
 *
 * Input sample types are chosen by `input_bits`:
 *   1, 2, 4  packed little-endian within bytes (sample k of a row lives in
 *            byte k / (8 / bits) at bit (k % (8 / bits)) * bits), unsigned,
 *   8        uint8_t,
 *   16       uint16_t,
 *   32       float.
 * Integer inputs are accumulated exactly in 32-bit integers and converted to
 * float once; float input is accumulated in float32 in channel order, which
 * is the reference's own order, so results equal the reference's bit for bit.
 */
#ifndef DEDISP_GB300_H
#define DEDISP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DD_ABI_VERSION 1

typedef enum dd_status {
  DD_OK = 0,
  DD_ERR_INVALID_ARGUMENT = -1, /* bad shape, null pointer, bad enum */
  DD_ERR_NO_DEVICE = -2,        /* no CUDA device visible */
  DD_ERR_CUDA = -3,             /* a CUDA runtime call failed */
  DD_ERR_OUT_OF_MEMORY = -4,    /* device allocation failed */
  DD_ERR_UNSUPPORTED = -5,      /* input bits / tile config not supported */
  DD_ERR_TIMEOUT = -6,          /* a bounded device-side wait ran out */
  DD_ERR_FILE = -7,             /* a file could not be opened or parsed */
  DD_ERR_OVER_BUDGET = -8,      /* a request exceeds the memory budget */
  DD_ERR_NOT_FOUND = -9         /* a lookup found nothing */
} dd_status;

typedef enum dd_mode {
  DD_SINGLE_STEP = 0, /* Dedispersion::dedispersion */
  DD_STEP_ONE = 1,    /* Dedispersion::subbandDedispersionStepOne */
  DD_STEP_TWO = 2     /* Dedispersion::subbandDedispersionStepTwo */
} dd_mode;

/*
 * Geometry of one observation batch.  Field-for-field the state the
 * reference reads through AstroData::Observation (getters listed at
 * include/Dedispersion.hpp:70-176 and src/Shifts.cpp:20-42).  Fields with a
 * `_subbanding` suffix are the values the reference reads with
 * `subbanding = true`.
 */
typedef struct dd_observation {
  uint32_t nr_beams;
  uint32_t nr_synthesized_beams;
  uint32_t nr_channels;
  uint32_t nr_subbands;                     /* 1 in single-step mode */
  uint32_t nr_samples_per_batch;            /* S  */
  uint32_t nr_samples_per_dispersed_batch;  /* S_disp >= S + max delay */
  uint32_t nr_samples_per_batch_subbanding; /* S1 (step one output length) */
  uint32_t nr_samples_per_dispersed_batch_subbanding; /* S1_disp */
  uint32_t nr_dms;
  uint32_t nr_dms_subbanding;
  uint32_t downsampling;                    /* must be 1 (AstroData default) */
  uint32_t nr_zapped_channels;              /* informational */
  float first_dm;
  float dm_step;
  float first_dm_subbanding;
  float dm_step_subbanding;
  float sampling_time;                      /* seconds */
  float min_freq;                           /* MHz, lowest channel */
  float channel_bandwidth;                  /* MHz */
} dd_observation;

/*
 * Tile configuration; field-for-field Dedispersion::DedispersionConf
 * (include/Dedispersion.hpp:34-54) plus the isa::OpenCL::KernelConf
 * threads/items it extends.  Meaning on the GPU:
 *   threads_d0  threads along time (32: one warp spans the time axis)
 *   threads_d1  warps along the DM axis
 *   items_d0    samples per thread (a multiple of 4)
 *   items_d1    DMs per thread
 *   unroll      channels staged per pipeline stage
 *   local_mem   1 = rows staged to shared memory by bulk copies (TMA)
 *   split_batches  kept for the tuned-file format; must be 0
 */
typedef struct dd_conf {
  uint32_t split_batches;
  uint32_t local_mem;
  uint32_t unroll;
  uint32_t threads_d0;
  uint32_t threads_d1;
  uint32_t threads_d2;
  uint32_t items_d0;
  uint32_t items_d1;
  uint32_t items_d2;
} dd_conf;

/* Row pitches and buffer sizes the reference's layout gives for one mode. */
typedef struct dd_layout {
  uint64_t input_row_bytes;   /* bytes between consecutive channel rows */
  uint64_t input_bytes;       /* whole input buffer */
  uint64_t output_row_elems;  /* floats between consecutive DM rows */
  uint64_t output_bytes;      /* whole output buffer */
  uint64_t mapping_row_elems; /* uint32 per synthesized beam in beamMapping */
  uint64_t zapped_elems;      /* uint32 entries of the zapped mask */
  uint64_t shifts_elems;      /* floats of the shift table */
  uint32_t max_delay;         /* largest per-channel delay in samples */
  uint32_t required_dispersed_samples; /* S (or S1) + max_delay */
} dd_layout;

/* ---- library ------------------------------------------------------------ */

/* Message of the last error raised on this thread ("" if none). */
const char *dd_last_error(void);
/* DD_ABI_VERSION of the loaded library. */
int dd_version(void);
/* Number of visible CUDA devices (0 on a host without a GPU). */
dd_status dd_device_count(int *count);

/* ---- host geometry (no device needed) ----------------------------------- */

/* isa::utils::pad: round `value` up to a multiple of `padding` (0 = none). */
uint64_t dd_pad(uint64_t value, uint64_t padding);

/* Dedispersion::getShifts (src/Shifts.cpp:20-30): per-channel delay in
 * samples per unit DM; the table is pad(C, padding/4) floats, last channel
 * and padding zero.  `capacity` is the number of floats `shifts` holds. */
dd_status dd_get_shifts(const dd_observation *obs, uint32_t padding,
                        float *shifts, size_t capacity);

/* Dedispersion::getShiftsStepTwo (src/Shifts.cpp:32-42): per-subband delay
 * per unit DM, relative to the highest channel of each subband. */
dd_status dd_get_shifts_step_two(const dd_observation *obs, uint32_t padding,
                                 float *shifts, size_t capacity);

/* Observation frequency getters (AstroData::Observation). */
float dd_max_freq(const dd_observation *obs);
float dd_subband_min_freq(const dd_observation *obs);
float dd_subband_max_freq(const dd_observation *obs);
float dd_subband_bandwidth(const dd_observation *obs);

/* Buffer layout of one mode.  `shifts` may be NULL (max_delay is then 0). */
dd_status dd_get_layout(const dd_observation *obs, dd_mode mode,
                        uint32_t input_bits, uint32_t padding,
                        const float *shifts, dd_layout *layout);

/* Default tile configuration the engine picks for a mode and input type. */
dd_status dd_default_conf(const dd_observation *obs, dd_mode mode,
                          uint32_t input_bits, dd_conf *conf);

/* DedispersionConf::print (src/Dedispersion.cpp:87-89):
 * "split local unroll tD0 tD1 tD2 iD0 iD1 iD2".  Writes at most `capacity`
 * bytes including the terminating NUL. */
dd_status dd_conf_print(const dd_conf *conf, char *text, size_t capacity);

/* readTunedDedispersionConf (src/Dedispersion.cpp:20-81): look up the entry
 * for (`device`, `nr_dms`) in a tuned-configuration text file whose lines
 * read "device nrDMs split local unroll tD0 tD1 tD2 iD0 iD1 iD2"; lines not
 * starting with a letter are ignored.  DD_ERR_FILE if the file cannot be
 * opened, DD_ERR_NOT_FOUND if no line matches. */
dd_status dd_read_tuned_conf(const char *path, const char *device,
                             uint32_t nr_dms, dd_conf *conf);

/* Append one line in the same format to `path`. */
dd_status dd_write_tuned_conf(const char *path, const char *device,
                              uint32_t nr_dms, const dd_conf *conf);

/* ---- synchronous host-buffer calls -------------------------------------- */
/* Drop-in replacements of the reference's CPU templates.  Host pointers in
 * the reference layout; the call copies to the device, runs, copies the
 * result back and returns when `output` holds it.  An `output` in pinned
 * host memory on a device that reaches host memory through the host's page
 * tables (a Grace host) is written by the kernels directly, without a copy
 * back; the result is the same. */

/* Dedispersion::dedispersion<I,L,O> (include/Dedispersion.hpp:59, 70-109). */
dd_status dd_dedispersion(const dd_observation *obs, const uint32_t *zapped,
                          const uint32_t *beam_mapping, const void *input,
                          float *output, const float *shifts,
                          uint32_t padding, uint32_t input_bits);

/* Dedispersion::subbandDedispersionStepOne (include/Dedispersion.hpp:60,
 * 111-153).  Output layout [beam][DM1][subband][pad(S1)]. */
dd_status dd_subband_dedispersion_step_one(const dd_observation *obs,
                                           const uint32_t *zapped,
                                           const void *input, float *output,
                                           const float *shifts,
                                           uint32_t padding,
                                           uint32_t input_bits);

/* Dedispersion::subbandDedispersionStepTwo (include/Dedispersion.hpp:61,
 * 155-176).  Float input [beam][DM1][subband][pad(S1)], output
 * [synthesized beam][DM1 * DM2][pad(S)]. */
dd_status dd_subband_dedispersion_step_two(const dd_observation *obs,
                                           const uint32_t *beam_mapping,
                                           const float *input, float *output,
                                           const float *shifts,
                                           uint32_t padding);

/* ---- subband pipeline: step one then step two on the device ------------- */
/* No counterpart in the reference, which runs the two steps as separate calls
 * (the two declarations above) with a float intermediate.  A pipeline owns
 * the intermediate.  When every subband's step-one sums fit 16 bits (live
 * channels per subband x (2^bits - 1) <= 65535) it is packed, one 32-bit
 * word per sample holding two coarse DMs' exact sums: half the bytes, and
 * step two adds both with one load.  Otherwise it runs the two float steps.
 * The output equals step one followed by step two bit for bit, in step two's
 * layout [synthesized beam][DM1 * DM2][pad(S)]; input in step one's. */
typedef struct dd_subband dd_subband;
dd_status dd_subband_create(dd_subband **pipeline, const dd_observation *obs,
                            uint32_t input_bits, uint32_t padding, int device);
/* Shift tables of both steps (getShifts, getShiftsStepTwo), the zapped mask
 * (step one) and the beam mapping (step two); builds both steps' tables. */
dd_status dd_subband_set_tables(dd_subband *pipeline, const float *shifts,
                                size_t n_shifts, const float *shifts_step_two,
                                size_t n_shifts_step_two,
                                const uint32_t *zapped, size_t n_zapped,
                                const uint32_t *beam_mapping, size_t n_mapping);
/* Enqueue both steps on `stream` (device pointers). */
dd_status dd_subband_run(dd_subband *pipeline, const void *d_input,
                         float *d_output, void *stream);
/* Synchronize `stream` and report a device-side timeout of either step. */
dd_status dd_subband_check(dd_subband *pipeline, void *stream);
/* Whether the intermediate is packed, and its device bytes. */
dd_status dd_subband_info(const dd_subband *pipeline, int *packed,
                          uint64_t *intermediate_bytes);
/* enable = 1: step one of each run is launched as a programmatic dependent of
 * the kernel before it on the stream (dd_plan_set_overlap), so that it starts
 * while the previous run's step two finishes; it writes the intermediate only
 * after that step two completed.  Only for runs whose input the kernel before
 * them does not write.  Off by default. */
dd_status dd_subband_set_overlap(dd_subband *pipeline, int enable);
/* chunks >= 2: each run splits step two's time tiles into `chunks` ranges and
 * launches each range right after the step-one tiles it reads (its samples
 * plus the largest step-two delay), step one on a stream of the pipeline's
 * own one range ahead, so that the intermediate is read back from L2 rather
 * than from device memory.  0 or 1 (the default): each step over all its
 * tiles in one launch.  Results are the same bit for bit; the overlap flag
 * does not apply to chunked runs. */
dd_status dd_subband_set_chunks(dd_subband *pipeline, int chunks);
/* Tile configuration of the packed step two (0 .. count - 1; 0 default). */
dd_status dd_subband_set_pair_kernel(dd_subband *pipeline, int index);
int dd_subband_pair_kernel_count(void);
dd_status dd_subband_destroy(dd_subband *pipeline);
/* Both steps on host buffers, synchronously (input as for step one, output
 * as for step two; the intermediate never leaves the device). */
dd_status dd_subband_dedispersion(const dd_observation *obs,
                                  const uint32_t *zapped,
                                  const uint32_t *beam_mapping,
                                  const void *input, float *output,
                                  const float *shifts,
                                  const float *shifts_step_two,
                                  uint32_t padding, uint32_t input_bits);

/* Single-step dedispersion that allocates no device memory.  It has no
 * counterpart in the reference.  It is for callers that cannot call
 * cudaMalloc where they dedisperse: a real-time loop that must not block
 * (cudaMalloc/cudaFree can synchronize the device), or a framework that owns
 * all device memory through its own capped pool.  The caller passes device
 * input and output buffers in the layout of dd_dedispersion and host tables;
 * the engine's descriptor tables and status word live in one fixed file-scope
 * device array of about 1 MiB that every GPU loading the library keeps until
 * exit.  Limits: at most 4096 synthesized beams and 61440 live rows
 * (synthesized beams x non-zapped channels); larger requests return
 * DD_ERR_UNSUPPORTED.  The call enqueues on `stream` (a cudaStream_t of the
 * current device; another device's stream is DD_ERR_INVALID_ARGUMENT) and
 * waits on it until the output is complete.  The first call on a device
 * looks up the array's address, so that first call should come before any
 * stream capture begins.  All calls share the array, so calls that overlap
 * on the GPU race (host threads are serialized inside the call). */
dd_status dd_dedispersion_noalloc(const dd_observation *obs,
                                  const uint32_t *zapped,
                                  const uint32_t *beam_mapping,
                                  const void *d_input, float *d_output,
                                  const float *shifts, uint32_t padding,
                                  uint32_t input_bits, void *stream);

/* ---- plans: device-resident tables, asynchronous device-pointer runs ---- */
/* The device twins of the generated OpenCL kernels `dedispersion`,
 * `dedispersionStepOne`, `dedispersionStepTwo` (include/Dedispersion.hpp:
 * 203-540, 543-882, 884-1122), launched as src/DedispersionTest.cpp:366-399
 * launches them.  A plan owns its device tables; the caller owns the data
 * buffers.  A plan is used from one thread/stream at a time; distinct plans
 * are independent. */
typedef struct dd_plan dd_plan;

/* `conf` may be NULL: the default kernel of the shape (dd_default_conf), or
 * where its tile does not fit the shape, the direct default and then the
 * other direct tiles of the input width, largest first.  For single-step
 * 1-8-bit input the default is the shared-partial-sum tile while its
 * executed adds stay below 0.34 of the direct sum, else the direct default
 * (measured crossover).  For single-step float input it is the TMEM-window
 * tile (items_d2 = 3; same float order as the scalar tile, bit-identical)
 * where 16 DMs move a row's delay by at most 45 samples, else the scalar
 * tile.  `device` is a CUDA device index. */
dd_status dd_plan_create(dd_plan **plan, const dd_observation *obs,
                         dd_mode mode, uint32_t input_bits, uint32_t padding,
                         const dd_conf *conf, int device);
/* Host tables, copied to the device when the plan is first used (run,
 * timing, dd_plan_adds).  Shifts are required; the zapped mask (nonzero =
 * skip) defaults to none zapped, the beam mapping to identity. */
dd_status dd_plan_set_shifts(dd_plan *plan, const float *shifts, size_t n);
dd_status dd_plan_set_zapped(dd_plan *plan, const uint32_t *zapped, size_t n);
dd_status dd_plan_set_beam_mapping(dd_plan *plan, const uint32_t *mapping,
                                   size_t n);
/* Compiled tile configurations: how many, and each one's name, input
 * element width (8 = the 1/2/4/8-bit family) and DedispersionConf. */
int dd_kernel_count(void);
dd_status dd_kernel_info(int index, char *name, size_t capacity,
                         uint32_t *elem_bits, dd_conf *conf);
/* dd_plan_create with compiled configuration `kernel_index` (the tuner's
 * entry point: it enumerates configurations by index). */
dd_status dd_plan_create_with_kernel(dd_plan **plan, const dd_observation *obs,
                                     dd_mode mode, uint32_t input_bits,
                                     uint32_t padding, int kernel_index,
                                     int device);
/* Enqueue one run on `stream` (a cudaStream_t; NULL = legacy default).
 * Device pointers in the layout dd_get_layout describes; returns after the
 * launch is queued. */
dd_status dd_plan_run(dd_plan *plan, const void *d_input, float *d_output,
                      void *stream);
/* Synchronize `stream` and report any device-side error the plan recorded
 * (DD_ERR_TIMEOUT for an expired bounded wait). */
dd_status dd_plan_check(dd_plan *plan, void *stream);
/* Kernel launches one dd_plan_run enqueues. */
dd_status dd_plan_launches(const dd_plan *plan, uint32_t *launches);
/* The configuration the plan runs with. */
dd_status dd_plan_get_conf(const dd_plan *plan, dd_conf *conf);
/* Integer adds one dd_plan_run performs, tile padding included: rows x DMs x
 * samples for the direct-sum kernels; partial sums plus series adds for the
 * shared-partial-sum kernels (configurations with items_d2 = 8), which reach
 * the same sums with fewer adds.  No reference counterpart. */
dd_status dd_plan_adds(const dd_plan *plan, uint64_t *adds);
/* enable = 1: each dd_plan_run of this plan is launched as a programmatic
 * dependent of the previous kernel on its stream, so that its tiles start on
 * SMs the previous launch's last wave leaves idle; the kernel waits for the
 * previous launch to complete before it writes anything.  Only for runs whose
 * input is not written by the kernel launched just before them on the stream
 * (consecutive independent batches).  Applies to the shared-partial-sum and
 * 1/2/4/8-bit direct kernels; the 16-bit and float kernels (scalar and
 * TMEM-window) launch as usual.
 * Off by default. */
/* Limit, in nanoseconds, of each bounded device-side wait for a staged
 * copy in this plan's runs (0, the default: 2 s).  When a wait runs out the
 * kernel stops its tile, lets the copies it has in flight land, and the next
 * dd_plan_check returns DD_ERR_TIMEOUT; the context stays usable.  A limit
 * below 1000 ns gives up as soon as the first test finds a copy not yet
 * landed: that exercises the path without a fault (the test of the timeout
 * handling uses 1 ns); production code leaves the limit at 0.  No
 * counterpart in the reference, whose host code reports OpenCL errors
 * (src/DedispersionTuning.cpp:396-409). */
dd_status dd_plan_set_wait_limit(dd_plan *plan, uint32_t ns);
dd_status dd_plan_set_overlap(dd_plan *plan, int enable);
dd_status dd_plan_destroy(dd_plan *plan);

/* ---- detection statistics of the output, computed in the same pass ------ */
/* No counterpart in the reference: its output goes to the next program of a
 * pipeline (an S/N search per DM), which reads the DM-time plane back from
 * memory.  For single-step plans on input of 1-16 bits (integer sums), per
 * output row (synthesized beam x DM): the exact sum and sum of squares of its
 * samples and its largest sample, the earliest on ties.  The
 * shared-partial-sum kernel accumulates them from its registers while it
 * writes the row; the other kernels take one extra pass over the output. */
typedef struct dd_dm_accum {
  uint64_t sum;     /* sum of the row's samples */
  uint64_t sum_sq;  /* sum of their squares */
  uint64_t peak;    /* largest sample << 32 | (0xffffffff - its sample index) */
} dd_dm_accum;
typedef struct dd_dm_stats {
  double mean;
  double stddev;         /* population standard deviation */
  double snr;            /* (peak - mean) / stddev; 0 when stddev is 0 */
  float peak;
  uint32_t peak_sample;
} dd_dm_stats;
/* dd_plan_run, and d_accum[beams x DMs] (device array, row = synthesized beam
 * * nr_dms + DM) set to the statistics of the output it writes.  The call
 * clears d_accum on `stream` first. */
dd_status dd_plan_run_stats(dd_plan *plan, const void *d_input, float *d_output,
                            dd_dm_accum *d_accum, void *stream);
/* Host: mean, standard deviation, peak, its sample and S/N of `rows` rows of
 * `samples` samples from their accumulators. */
dd_status dd_dm_stats_from_accum(const dd_dm_accum *accum, size_t rows, uint32_t samples,
                                 dd_dm_stats *stats);

/* ---- ingest: SIGPROC filterbank and PSRDADA files ------------------------- */
/* The reference reads its input through AstroData's readers (ReadData, an
 * external dependency, CMakeLists.txt:8-15); these are the SIGPROC filterbank
 * and PSRDADA paths of that role, with the time-major to channel-row
 * transpose on the device. */
typedef struct dd_filterbank_info {
  uint32_t nchans, nbits, nifs, nbeams, ibeam, data_type;
  uint64_t nsamples;      /* from the header, else from the file size */
  uint64_t header_bytes;  /* offset of the first sample */
  double tsamp;           /* seconds */
  double fch1, foff;      /* MHz: first channel, channel step (< 0: descending) */
  double tstart, refdm;
  char source_name[80];
} dd_filterbank_info;
/* Parse the header of a SIGPROC filterbank file. */
dd_status dd_filterbank_info_read(const char *path, dd_filterbank_info *info);
/* Samples [start, start + count) of IF 0, time-major, into a host buffer of
 * count * nchans * nbits / 8 bytes. */
dd_status dd_filterbank_read(const char *path, const dd_filterbank_info *info,
                             uint64_t start, uint64_t count, void *time_major);
/* Channel count, lowest frequency, bandwidth and sampling time of `obs`
 * from the header: the engine's channel c is at min_freq + c * bandwidth, so
 * files with foff < 0 are read with their channels reversed. */
dd_status dd_filterbank_observation(const dd_filterbank_info *info, dd_observation *obs);
/* A PSRDADA file: an ASCII header of HDR_SIZE bytes ("KEY value" lines),
 * then the samples.  Detected filterbank data only: NPOL = 1, NDIM = 1,
 * ORDER TF or TFP (time-major), NBIT 1/2/4/8/16/32. */
typedef struct dd_dada_info {
  uint32_t nchan, nbit, npol, ndim;
  uint64_t nsamples;      /* from the data bytes after the header */
  uint64_t header_bytes;  /* HDR_SIZE: offset of the first sample */
  uint64_t obs_offset;    /* OBS_OFFSET: bytes of the observation before this file */
  double tsamp;           /* seconds (TSAMP is in microseconds) */
  double freq, bw;        /* MHz: centre of the band, total bandwidth (< 0: descending) */
  char source[64];
  char utc_start[32];
} dd_dada_info;
/* Parse the header of a PSRDADA file. */
dd_status dd_dada_info_read(const char *path, dd_dada_info *info);
/* Samples [start, start + count), time-major, into a host buffer of
 * count * nchan * nbit / 8 bytes. */
dd_status dd_dada_read(const char *path, const dd_dada_info *info, uint64_t start,
                       uint64_t count, void *time_major);
/* Channel count, lowest channel centre, channel width and sampling time of
 * `obs` from the header (channel i of the file is centred at
 * freq - bw / 2 + (i + 0.5) * bw / nchan; bw < 0 files are reversed). */
dd_status dd_dada_observation(const dd_dada_info *info, dd_observation *obs);
/* Device: a time-major 8-bit block [count][nchans] into channel rows of a
 * plan's input (row c at d_dst + c * dst_row_bytes), at sample
 * dst_sample_offset of each row; `reverse` = 1 writes file channel c to row
 * nchans - 1 - c.  Asynchronous on `stream`. */
dd_status dd_transpose_time_major(const void *d_src, uint32_t count, uint32_t nchans,
                                  int reverse, void *d_dst, uint64_t dst_row_bytes,
                                  uint64_t dst_sample_offset, void *stream);

/* ---- batches: many beams in one graph launch ----------------------------- */
/* No counterpart in the reference (its driver launches one kernel per beam
 * set, src/DedispersionTest.cpp:366-399).  A batch holds single-step problems
 * of 1/2/4/8-bit input, each with its own geometry, tables and device
 * buffers; committing it records one CUDA graph that computes them all.  By
 * default the graph forks into a few concurrent branches of the problems' own
 * default kernels (as dd_plan_create with no configuration picks them;
 * longest first, balanced by tile cost).  The persistent form is one
 * work list over all the problems' tiles (longest first) run by a persistent
 * direct-tile kernel.  Results equal dd_plan_run's for each problem bit for
 * bit. */
typedef struct dd_batch dd_batch;
dd_status dd_batch_create(dd_batch **batch, int device);
/* Add one single-step problem; `index` (may be NULL) receives its position.
 * Host tables as for dd_dedispersion, device buffers as for dd_plan_run. */
dd_status dd_batch_add(dd_batch *batch, const dd_observation *obs,
                       uint32_t input_bits, uint32_t padding,
                       const float *shifts, const uint32_t *zapped,
                       const uint32_t *beam_mapping, const void *d_input,
                       float *d_output, uint32_t *index);
/* dd_batch_add with the problem's configuration chosen by the caller
 * (registry index `kernel`, dd_kernel_info; -1: the problem's default), for
 * the graph form: a tuner's per-problem pick.  A configuration that cannot
 * run the problem is DD_ERR_UNSUPPORTED and adds nothing.  No counterpart
 * in the reference, whose tuned configuration applies to one kernel launch
 * (src/Dedispersion.cpp:20-81). */
dd_status dd_batch_add_with_kernel(dd_batch *batch, const dd_observation *obs,
                                   uint32_t input_bits, uint32_t padding, const float *shifts,
                                   const uint32_t *zapped, const uint32_t *beam_mapping,
                                   const void *d_input, float *d_output, int kernel,
                                   uint32_t *index);
dd_status dd_batch_commit(dd_batch *batch);
/* Enqueue the batch on `stream`: replay the recorded graph (use_graph = 1)
 * or launch directly. */
dd_status dd_batch_run(dd_batch *batch, void *stream, int use_graph);
/* Synchronize `stream` and report a device-side timeout. */
dd_status dd_batch_check(dd_batch *batch, void *stream);
/* Problems and tiles of a committed batch, and its concurrent branches (graph
 * form) or persistent CTAs (persistent form). */
dd_status dd_batch_info(const dd_batch *batch, uint32_t *problems,
                        uint32_t *tiles, uint32_t *grid);
/* 1 if a committed batch runs in the graph form (each problem's own kernel),
 * 0 if in the persistent form. */
dd_status dd_batch_shared(const dd_batch *batch, int *shared);
/* enable = 1: commit in the persistent form (one persistent direct-tile
 * kernel over all the problems' tiles).  Takes effect at the next commit. */
dd_status dd_batch_set_persistent(dd_batch *batch, int enable);
dd_status dd_batch_destroy(dd_batch *batch);

/* ---- streams: one beam of a real-time batch stream ---------------------- */
/* No counterpart in the reference (its splitBatches mode is empty,
 * include/Dedispersion.hpp:202).  `obs` gives the per-batch geometry: S new
 * samples per batch (nr_samples_per_batch), one beam, the DM range(s) and, with
 * `subband` = 1, the subband fields of a step one -> step two pipeline.  The
 * stream keeps the max-delay tail of every channel on the device and each
 * push dedisperses [tail | new batch]: output k equals the plain path on
 * stream samples [k*S - tail, (k+1)*S) (zeros before the first batch). */
typedef struct dd_stream dd_stream;
/* Device bytes a stream of this geometry holds (for admission), and its tail. */
dd_status dd_stream_bytes(const dd_observation *obs, int subband,
                          uint32_t input_bits, uint32_t padding,
                          const float *shifts, const float *shifts_step_two,
                          const uint32_t *zapped, uint64_t *device_bytes,
                          uint32_t *tail);
dd_status dd_stream_create(dd_stream **stream, const dd_observation *obs,
                           int subband, uint32_t input_bits, uint32_t padding,
                           const float *shifts, const float *shifts_step_two,
                           const uint32_t *zapped, int device);
/* Pinned staging input [C][S samples] and pinned output [rows][S] of the
 * next push, device output in the plan layout. */
dd_status dd_stream_buffers(dd_stream *stream, void **h_input, float **h_output,
                            float **d_output);
dd_status dd_stream_info(const dd_stream *stream, uint32_t *tail,
                         uint64_t *device_bytes, uint64_t *input_row_bytes,
                         uint32_t *output_rows);
/* Enqueue one batch (the staging input) on `cuda_stream`: copy in, dedisperse,
 * copy the output to the pinned output, carry the tail.  Refill the staging
 * input only after the previous push completed. */
dd_status dd_stream_push(dd_stream *stream, void *cuda_stream);
/* From now on take each batch as a time-major 8-bit block [S][C] in the
 * staging input (file order of SIGPROC and PSRDADA data; `reverse` = 1 when
 * the file's channel 0 is the highest frequency): a push copies the block to
 * the device and transposes it into the ring (dd_transpose_time_major).
 * Adds S * C device bytes.  8-bit streams only. */
dd_status dd_stream_set_time_major(dd_stream *stream, int reverse);
/* enable = 1: two pinned staging/output pairs used in turn (push k uses pair
 * k % 2), so that the next batch can be staged, and the previous output read,
 * while a push is in flight; dd_stream_buffers returns the next push's pair.
 * A pair may be refilled once the push that used it completed. */
dd_status dd_stream_set_double_buffer(dd_stream *stream, int enable);
/* Pair `index` (0 or 1) of the staging input and pinned output, and the
 * index the next push uses. */
dd_status dd_stream_buffer(dd_stream *stream, int index, void **h_input, float **h_output);
dd_status dd_stream_next_buffer(const dd_stream *stream, int *index);
dd_status dd_stream_destroy(dd_stream *stream);

/* ---- learned tuning: the cost model's network ---------------------------- */
/* No counterpart in the reference (its tuner is an exhaustive sweep,
 * src/DedispersionTuning.cpp:201-437, which stays the arbiter of what is fastest).  An MLP
 * in -> hidden x hidden_layers -> 1 with ReLU, bf16 weights (fp32 master copy
 * for Adam), fp32 accumulation, MSE loss, trained and run by the library's own
 * CUDA kernels.  Parameters are exchanged as flat fp32 arrays: per layer
 * W [out][in] then b [out]. */
typedef struct dd_mlp dd_mlp;
dd_status dd_mlp_create(dd_mlp **mlp, uint32_t in_features, uint32_t hidden,
                        uint32_t hidden_layers, uint64_t seed, int device);
dd_status dd_mlp_param_count(const dd_mlp *mlp, uint64_t *count);
dd_status dd_mlp_get_params(dd_mlp *mlp, float *params, uint64_t count);
dd_status dd_mlp_set_params(dd_mlp *mlp, const float *params, uint64_t count);
/* Predictions for `n` rows of features (host arrays). */
dd_status dd_mlp_forward(dd_mlp *mlp, const float *x, uint32_t n, float *y);
/* MSE loss and its gradient w.r.t. every parameter (host arrays). */
dd_status dd_mlp_gradients(dd_mlp *mlp, const float *x, const float *target,
                           uint32_t n, float *grad, float *loss);
/* `steps` full-batch Adam steps at learning rate `lr`; final loss out. */
dd_status dd_mlp_train(dd_mlp *mlp, const float *x, const float *target,
                       uint32_t n, uint32_t steps, float lr, float *final_loss);
dd_status dd_mlp_destroy(dd_mlp *mlp);

/* ---- tuning support ------------------------------------------------------ */
/* Measured add throughput of device `device`: streams of independent
 * float adds and of 32-bit integer adds on every SM, timed with CUDA events,
 * best of `repeats` runs (after one warm-up run); results in adds per second.
 * It is the denominator of the path's add roofline (the direct sum is bound
 * by adds, not by HBM).  No counterpart in the reference. */
dd_status dd_measure_add_rate(int device, uint32_t repeats, double *fadd_per_s,
                              double *iadd_per_s);

/* Mean device time of `iterations` runs of a plan after `warmup` runs, timed
 * with CUDA events on a private stream (the reference's tuner times
 * enqueue + wait with a host timer, src/DedispersionTuning.cpp:384-395). */
dd_status dd_plan_time(dd_plan *plan, const void *d_input, float *d_output,
                       uint32_t warmup, uint32_t iterations, float *mean_ms,
                       float *std_ms);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* DEDISP_GB300_H */

// dd_ingest.cu -- SIGPROC filterbank and PSRDADA input: header parsing,
// block reads and the device transpose from the files' time-major samples to
// the engine's channel rows.
//
// The reference reads its input through AstroData's readers (ReadData, an
// external dependency named in its CMakeLists.txt:8-15 and absent from its
// tree).  The SIGPROC filterbank format is restated here from its published
// definition: a header of keywords, each an int32 length and that many
// characters, between "HEADER_START" and "HEADER_END"; integer keywords carry
// an int32 value, floating keywords a float64, string keywords a length-
// prefixed string; then the samples, time-major: for each time sample, for
// each IF, nchans channel values of nbits bits, the first channel at fch1 and
// the next ones foff MHz apart (foff < 0 in most files: descending).
//
// The PSRDADA file format is restated from its published definition as well:
// an ASCII header of HDR_SIZE bytes (4096 by default), one "KEY value" per
// line and NUL-padded, then the data.  For detected filterbank data (NPOL 1,
// NDIM 1) in time-major order (ORDER TF or TFP) each time sample holds NCHAN
// values of NBIT bits; the band of BW MHz (negative: channel 0 highest) is
// centred at FREQ MHz; TSAMP is in microseconds.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>

#include "../../include/dedisp_gb300.h"

namespace dd {
void set_last_error(const char *message);
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

bool read_string(std::ifstream &in, std::string *s) {
  int32_t n = 0;
  if (!in.read(reinterpret_cast<char *>(&n), 4) || n <= 0 || n > 4096) return false;
  s->resize((size_t)n);
  return static_cast<bool>(in.read(&(*s)[0], n));
}

// Keyword value kinds of the SIGPROC header.
enum Kind { kInt, kDouble, kString, kUnknown };

Kind kind_of(const std::string &k) {
  static const char *ints[] = {"telescope_id", "machine_id", "data_type", "barycentric",
                               "pulsarcentric", "nbits",     "nsamples",  "nchans",
                               "nifs",         "nbeams",     "ibeam",     nullptr};
  static const char *dbls[] = {"az_start", "za_start", "src_raj", "src_dej", "tstart",
                               "tsamp",    "fch1",     "foff",    "refdm",   "period",
                               "refrm",    nullptr};
  static const char *strs[] = {"source_name", "rawdatafile", nullptr};
  for (int i = 0; ints[i]; i++)
    if (k == ints[i]) return kInt;
  for (int i = 0; dbls[i]; i++)
    if (k == dbls[i]) return kDouble;
  for (int i = 0; strs[i]; i++)
    if (k == strs[i]) return kString;
  return kUnknown;
}

// Tiled transpose of a time-major 8-bit block [count][nchans] into channel
// rows: dst[(chan') * row_bytes + offset + t] = src[t * nchans + chan], with
// chan' = nchans - 1 - chan when the channels are reversed.  32 x 32 tiles
// through shared memory: both the reads and the writes are coalesced.
__global__ void transpose8_kernel(const uint8_t *__restrict__ src, uint32_t count,
                                  uint32_t nchans, int reverse, uint8_t *__restrict__ dst,
                                  uint64_t row_bytes, uint64_t offset) {
  __shared__ uint8_t tile[32][33];
  const uint32_t t0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  const uint32_t tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (uint32_t k = ty; k < 32; k += 8) {
    const uint32_t t = t0 + k, c = c0 + tx;
    tile[k][tx] = (t < count && c < nchans) ? src[(uint64_t)t * nchans + c] : 0;
  }
  __syncthreads();
  for (uint32_t k = ty; k < 32; k += 8) {
    const uint32_t c = c0 + k, t = t0 + tx;
    if (c < nchans && t < count) {
      const uint32_t row = reverse ? nchans - 1 - c : c;
      dst[(uint64_t)row * row_bytes + offset + t] = tile[tx][k];
    }
  }
}

// Reads the "KEY value" lines of a PSRDADA header of `bytes` bytes.
bool dada_keys(std::ifstream &in, uint64_t bytes, std::map<std::string, std::string> *keys) {
  std::string text(bytes, '\0');
  in.seekg(0);
  if (!in.read(&text[0], (std::streamsize)bytes)) return false;
  text.resize(std::strlen(text.c_str()));  // NUL padding ends the header
  std::istringstream lines(text);
  std::string line;
  while (std::getline(lines, line)) {
    const size_t a = line.find_first_not_of(" \t\r");
    if (a == std::string::npos || line[a] == '#') continue;
    const size_t b = line.find_first_of(" \t", a);
    if (b == std::string::npos) continue;
    const size_t c = line.find_first_not_of(" \t", b);
    if (c == std::string::npos) continue;
    size_t e = line.find_last_not_of(" \t\r");
    (*keys)[line.substr(a, b - a)] = line.substr(c, e + 1 - c);
  }
  return true;
}

// Word-wide transpose for 4-byte aligned blocks (nchans, the row pitch and
// the sample offset multiples of 4): 64 samples x 64 channels per CTA of 256
// threads.  Loads and stores are 32-bit and coalesced (16 words per time row
// or channel row); each thread transposes a 4 x 4 byte block (4 samples x 4
// channels) in registers with byte permutes.
__global__ void __launch_bounds__(256) transpose8x4_kernel(
    const uint32_t *__restrict__ src, uint32_t count, uint32_t nchans, int reverse,
    uint8_t *__restrict__ dst, uint64_t row_bytes, uint64_t offset) {
  __shared__ uint32_t tile[64][17];  // [sample][channel word], padded
  const uint32_t t0 = blockIdx.x * 64, c0 = blockIdx.y * 64;
  const uint32_t tid = threadIdx.x, cwords = nchans / 4;
#pragma unroll
  for (uint32_t j = 0; j < 4; j++) {
    const uint32_t r = tid / 16 + 16 * j, col = tid % 16;
    const uint32_t t = t0 + r, cw = c0 / 4 + col;
    tile[r][col] = (t < count && cw < cwords) ? src[(uint64_t)t * cwords + cw] : 0u;
  }
  __syncthreads();
  // One 4 x 4 byte block per thread: sample word sw (samples 4 sw .. +3) of
  // channel word cword (channels 4 cword .. +3); 16 x 16 blocks per tile.
  const uint32_t sw = tid % 16, cword = tid / 16;
  const uint32_t w0 = tile[4 * sw][cword], w1 = tile[4 * sw + 1][cword];
  const uint32_t w2 = tile[4 * sw + 2][cword], w3 = tile[4 * sw + 3][cword];
  // w_k = channels 4 cword .. +3 of sample 4 sw + k; out[m] = channel m's
  // four samples
  const uint32_t a = __byte_perm(w0, w1, 0x5140), b = __byte_perm(w0, w1, 0x7362);
  const uint32_t c = __byte_perm(w2, w3, 0x5140), d = __byte_perm(w2, w3, 0x7362);
  const uint32_t out[4] = {__byte_perm(a, c, 0x5410), __byte_perm(a, c, 0x7632),
                           __byte_perm(b, d, 0x5410), __byte_perm(b, d, 0x7632)};
  const uint32_t t = t0 + 4 * sw;
  if (t >= count) return;
#pragma unroll
  for (uint32_t m = 0; m < 4; m++) {
    const uint32_t ch = c0 + 4 * cword + m;
    if (ch >= nchans) break;
    const uint32_t row = reverse ? nchans - 1 - ch : ch;
    uint8_t *p = dst + (uint64_t)row * row_bytes + offset + t;
    if (t + 3 < count) {
      *reinterpret_cast<uint32_t *>(p) = out[m];
    } else {
      for (uint32_t k = 0; t + k < count; k++) p[k] = (uint8_t)(out[m] >> (8 * k));
    }
  }
}

}  // namespace

extern "C" {

dd_status dd_filterbank_info_read(const char *path, dd_filterbank_info *info) {
  if (!path || !info) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  std::memset(info, 0, sizeof(*info));
  info->nifs = 1;
  info->nbeams = 1;
  std::ifstream in(path, std::ios::binary);
  if (!in) return fail(DD_ERR_FILE, "Impossible to open %s", path);
  std::string key;
  if (!read_string(in, &key) || key != "HEADER_START")
    return fail(DD_ERR_FILE, "%s: not a SIGPROC filterbank (no HEADER_START)", path);
  bool have_nsamples = false;
  for (;;) {
    if (!read_string(in, &key)) return fail(DD_ERR_FILE, "%s: truncated header", path);
    if (key == "HEADER_END") break;
    const Kind k = kind_of(key);
    if (k == kInt) {
      int32_t v = 0;
      if (!in.read(reinterpret_cast<char *>(&v), 4))
        return fail(DD_ERR_FILE, "%s: truncated value of %s", path, key.c_str());
      if (key == "nbits") info->nbits = (uint32_t)v;
      else if (key == "nchans") info->nchans = (uint32_t)v;
      else if (key == "nifs") info->nifs = (uint32_t)v;
      else if (key == "nbeams") info->nbeams = (uint32_t)v;
      else if (key == "ibeam") info->ibeam = (uint32_t)v;
      else if (key == "data_type") info->data_type = (uint32_t)v;
      else if (key == "nsamples") { info->nsamples = (uint64_t)(uint32_t)v; have_nsamples = true; }
    } else if (k == kDouble) {
      double v = 0;
      if (!in.read(reinterpret_cast<char *>(&v), 8))
        return fail(DD_ERR_FILE, "%s: truncated value of %s", path, key.c_str());
      if (key == "tsamp") info->tsamp = v;
      else if (key == "fch1") info->fch1 = v;
      else if (key == "foff") info->foff = v;
      else if (key == "tstart") info->tstart = v;
      else if (key == "refdm") info->refdm = v;
    } else if (k == kString) {
      std::string v;
      if (!read_string(in, &v))
        return fail(DD_ERR_FILE, "%s: truncated value of %s", path, key.c_str());
      if (key == "source_name")
        std::snprintf(info->source_name, sizeof(info->source_name), "%s", v.c_str());
    } else {
      return fail(DD_ERR_FILE, "%s: unknown header keyword '%s'", path, key.c_str());
    }
  }
  info->header_bytes = (uint64_t)in.tellg();
  if (info->nchans == 0 || info->nifs == 0 ||
      (info->nbits != 1 && info->nbits != 2 && info->nbits != 4 && info->nbits != 8 &&
       info->nbits != 16 && info->nbits != 32))
    return fail(DD_ERR_FILE, "%s: nchans %u, nifs %u, nbits %u not supported", path,
                info->nchans, info->nifs, info->nbits);
  in.seekg(0, std::ios::end);
  const uint64_t data = (uint64_t)in.tellg() - info->header_bytes;
  const uint64_t bits_per_sample = (uint64_t)info->nchans * info->nifs * info->nbits;
  if (bits_per_sample % 8) return fail(DD_ERR_FILE, "%s: a time sample is not whole bytes", path);
  const uint64_t from_size = data / (bits_per_sample / 8);
  if (!have_nsamples || info->nsamples > from_size) info->nsamples = from_size;
  return DD_OK;
}

dd_status dd_filterbank_read(const char *path, const dd_filterbank_info *info, uint64_t start,
                             uint64_t count, void *time_major) {
  if (!path || !info || (!time_major && count)) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (start + count > info->nsamples)
    return fail(DD_ERR_INVALID_ARGUMENT, "samples [%llu, %llu) past the file's %llu",
                (unsigned long long)start, (unsigned long long)(start + count),
                (unsigned long long)info->nsamples);
  std::ifstream in(path, std::ios::binary);
  if (!in) return fail(DD_ERR_FILE, "Impossible to open %s", path);
  const uint64_t if_bytes = (uint64_t)info->nchans * info->nbits / 8;
  const uint64_t sample_bytes = if_bytes * info->nifs;
  char *dst = static_cast<char *>(time_major);
  if (info->nifs == 1) {
    in.seekg((std::streamoff)(info->header_bytes + start * sample_bytes));
    if (!in.read(dst, (std::streamsize)(count * sample_bytes)))
      return fail(DD_ERR_FILE, "%s: short read", path);
    return DD_OK;
  }
  for (uint64_t t = 0; t < count; t++) {  // IF 0 of each time sample
    in.seekg((std::streamoff)(info->header_bytes + (start + t) * sample_bytes));
    if (!in.read(dst + t * if_bytes, (std::streamsize)if_bytes))
      return fail(DD_ERR_FILE, "%s: short read", path);
  }
  return DD_OK;
}

dd_status dd_filterbank_observation(const dd_filterbank_info *info, dd_observation *obs) {
  if (!info || !obs) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (info->foff == 0) return fail(DD_ERR_INVALID_ARGUMENT, "foff is 0");
  // The engine's channel c is at min_freq + c * bandwidth (ascending).
  const double lowest = info->foff < 0 ? info->fch1 + (info->nchans - 1) * info->foff : info->fch1;
  obs->nr_channels = info->nchans;
  obs->min_freq = (float)lowest;
  obs->channel_bandwidth = (float)std::fabs(info->foff);
  obs->sampling_time = (float)info->tsamp;
  return DD_OK;
}

dd_status dd_dada_info_read(const char *path, dd_dada_info *info) {
  if (!path || !info) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  std::memset(info, 0, sizeof(*info));
  std::ifstream in(path, std::ios::binary);
  if (!in) return fail(DD_ERR_FILE, "Impossible to open %s", path);
  in.seekg(0, std::ios::end);
  const uint64_t size = (uint64_t)in.tellg();
  std::map<std::string, std::string> keys;
  if (size < 16 || !dada_keys(in, std::min<uint64_t>(size, 4096), &keys))
    return fail(DD_ERR_FILE, "%s: truncated PSRDADA header", path);
  if (!keys.count("HDR_SIZE")) return fail(DD_ERR_FILE, "%s: not a PSRDADA file (no HDR_SIZE)", path);
  const uint64_t hdr = std::strtoull(keys["HDR_SIZE"].c_str(), nullptr, 10);
  if (hdr == 0 || hdr > size) return fail(DD_ERR_FILE, "%s: HDR_SIZE %llu past the file", path,
                                          (unsigned long long)hdr);
  if (hdr > 4096) {
    keys.clear();
    if (!dada_keys(in, hdr, &keys)) return fail(DD_ERR_FILE, "%s: truncated PSRDADA header", path);
  }
  for (const char *k : {"NCHAN", "NBIT", "TSAMP", "FREQ", "BW"})
    if (!keys.count(k)) return fail(DD_ERR_FILE, "%s: PSRDADA header has no %s", path, k);
  auto u32 = [&](const char *k, uint32_t def) {
    return keys.count(k) ? (uint32_t)std::strtoul(keys[k].c_str(), nullptr, 10) : def;
  };
  info->header_bytes = hdr;
  info->nchan = u32("NCHAN", 0);
  info->nbit = u32("NBIT", 0);
  info->npol = u32("NPOL", 1);
  info->ndim = u32("NDIM", 1);
  info->obs_offset = keys.count("OBS_OFFSET") ? std::strtoull(keys["OBS_OFFSET"].c_str(), nullptr, 10) : 0;
  info->tsamp = std::strtod(keys["TSAMP"].c_str(), nullptr) * 1e-6;
  info->freq = std::strtod(keys["FREQ"].c_str(), nullptr);
  info->bw = std::strtod(keys["BW"].c_str(), nullptr);
  if (keys.count("SOURCE"))
    std::snprintf(info->source, sizeof(info->source), "%s", keys["SOURCE"].c_str());
  if (keys.count("UTC_START"))
    std::snprintf(info->utc_start, sizeof(info->utc_start), "%s", keys["UTC_START"].c_str());
  const std::string order = keys.count("ORDER") ? keys["ORDER"] : "TF";
  if (info->npol != 1 || info->ndim != 1 || (order != "TF" && order != "TFP"))
    return fail(DD_ERR_UNSUPPORTED,
                "%s: NPOL %u, NDIM %u, ORDER %s: detected time-major data only (NPOL 1, NDIM 1, "
                "ORDER TF)", path, info->npol, info->ndim, order.c_str());
  if (info->nchan == 0 ||
      (info->nbit != 1 && info->nbit != 2 && info->nbit != 4 && info->nbit != 8 &&
       info->nbit != 16 && info->nbit != 32))
    return fail(DD_ERR_FILE, "%s: NCHAN %u, NBIT %u not supported", path, info->nchan, info->nbit);
  const uint64_t bits_per_sample = (uint64_t)info->nchan * info->nbit;
  if (bits_per_sample % 8) return fail(DD_ERR_FILE, "%s: a time sample is not whole bytes", path);
  info->nsamples = (size - hdr) / (bits_per_sample / 8);
  return DD_OK;
}

dd_status dd_dada_read(const char *path, const dd_dada_info *info, uint64_t start, uint64_t count,
                       void *time_major) {
  if (!path || !info || (!time_major && count)) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (start + count > info->nsamples)
    return fail(DD_ERR_INVALID_ARGUMENT, "samples [%llu, %llu) past the file's %llu",
                (unsigned long long)start, (unsigned long long)(start + count),
                (unsigned long long)info->nsamples);
  std::ifstream in(path, std::ios::binary);
  if (!in) return fail(DD_ERR_FILE, "Impossible to open %s", path);
  const uint64_t sample_bytes = (uint64_t)info->nchan * info->nbit / 8;
  in.seekg((std::streamoff)(info->header_bytes + start * sample_bytes));
  if (!in.read(static_cast<char *>(time_major), (std::streamsize)(count * sample_bytes)))
    return fail(DD_ERR_FILE, "%s: short read", path);
  return DD_OK;
}

dd_status dd_dada_observation(const dd_dada_info *info, dd_observation *obs) {
  if (!info || !obs) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (info->bw == 0 || info->nchan == 0) return fail(DD_ERR_INVALID_ARGUMENT, "BW or NCHAN is 0");
  const double width = std::fabs(info->bw) / info->nchan;
  obs->nr_channels = info->nchan;
  obs->min_freq = (float)(info->freq - std::fabs(info->bw) / 2 + 0.5 * width);
  obs->channel_bandwidth = (float)width;
  obs->sampling_time = (float)info->tsamp;
  return DD_OK;
}

dd_status dd_transpose_time_major(const void *d_src, uint32_t count, uint32_t nchans,
                                  int reverse, void *d_dst, uint64_t dst_row_bytes,
                                  uint64_t dst_sample_offset, void *stream) {
  if (!d_src || !d_dst) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (dst_sample_offset + count > dst_row_bytes)
    return fail(DD_ERR_INVALID_ARGUMENT, "samples [%llu, %llu) past rows of %llu bytes",
                (unsigned long long)dst_sample_offset,
                (unsigned long long)(dst_sample_offset + count),
                (unsigned long long)dst_row_bytes);
  if (count == 0 || nchans == 0) return DD_OK;
  const bool words = nchans % 4 == 0 && dst_row_bytes % 4 == 0 && dst_sample_offset % 4 == 0 &&
                     reinterpret_cast<uintptr_t>(d_src) % 4 == 0 &&
                     reinterpret_cast<uintptr_t>(d_dst) % 4 == 0;
  if (words) {
    const dim3 grid((count + 63) / 64, (nchans + 63) / 64);
    transpose8x4_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const uint32_t *>(d_src), count, nchans, reverse,
        static_cast<uint8_t *>(d_dst), dst_row_bytes, dst_sample_offset);
  } else {
    const dim3 grid((count + 31) / 32, (nchans + 31) / 32), block(32, 8);
    transpose8_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const uint8_t *>(d_src), count, nchans, reverse,
        static_cast<uint8_t *>(d_dst), dst_row_bytes, dst_sample_offset);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(DD_ERR_CUDA, "launch transpose: %s", cudaGetErrorString(e));
  return DD_OK;
}

}  // extern "C"

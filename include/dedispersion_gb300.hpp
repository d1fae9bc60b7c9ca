// dedispersion_gb300.hpp -- source-compatible C++ surface of the reference's
// dedispersion path, over the C ABI in dedisp_gb300.h.
//
// A program written against TRASAL/Dedispersion's CPU entry points switches
// by including this header instead of Observation.hpp / Shifts.hpp /
// Dedispersion.hpp and linking libdedisp_gb300.so.  Names, argument order
// and meaning follow the reference:
//   AstroData::Observation            (setters/getters the path reads)
//   Dedispersion::getShifts           src/Shifts.cpp:20-30
//   Dedispersion::getShiftsStepTwo    src/Shifts.cpp:32-42
//   Dedispersion::DedispersionConf    include/Dedispersion.hpp:34-54
//   Dedispersion::dedispersion        include/Dedispersion.hpp:59, 70-109
//   Dedispersion::subbandDedispersionStepOne  include/Dedispersion.hpp:60
//   Dedispersion::subbandDedispersionStepTwo  include/Dedispersion.hpp:61
//   Dedispersion::readTunedDedispersionConf   src/Dedispersion.cpp:20-81
// The three compute templates run on the GPU and return when `output` holds
// the result.  Where the reference has no error path, a failure of the GPU
// path throws Dedispersion::DedispersionError (std::runtime_error).
#pragma once

#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "dedisp_gb300.h"

namespace AstroData {

// Thrown by readTunedDedispersionConf when its file cannot be opened.
class FileError : public std::runtime_error {
 public:
  explicit FileError(const std::string &what) : std::runtime_error(what) {}
};

class Observation {
 public:
  Observation() {
    c_ = dd_observation{};
    c_.nr_beams = 1;
    c_.nr_synthesized_beams = 1;
    c_.nr_subbands = 1;
    c_.downsampling = 1;
  }
  void setNrBeams(unsigned int v) { c_.nr_beams = v; }
  void setNrSynthesizedBeams(unsigned int v) { c_.nr_synthesized_beams = v; }
  void setNrSamplesPerBatch(unsigned int v, bool subbanding = false) {
    (subbanding ? c_.nr_samples_per_batch_subbanding : c_.nr_samples_per_batch) = v;
  }
  void setNrSamplesPerDispersedBatch(unsigned int v, bool subbanding = false) {
    (subbanding ? c_.nr_samples_per_dispersed_batch_subbanding
                : c_.nr_samples_per_dispersed_batch) = v;
  }
  void setSamplingTime(float v) { c_.sampling_time = v; }
  void setFrequencyRange(unsigned int subbands, unsigned int channels, float minFreq,
                         float channelBandwidth) {
    c_.nr_subbands = subbands;
    c_.nr_channels = channels;
    c_.min_freq = minFreq;
    c_.channel_bandwidth = channelBandwidth;
  }
  void setDMRange(unsigned int nrDMs, float firstDM, float step, bool subbanding = false) {
    if (subbanding) {
      c_.nr_dms_subbanding = nrDMs;
      c_.first_dm_subbanding = firstDM;
      c_.dm_step_subbanding = step;
    } else {
      c_.nr_dms = nrDMs;
      c_.first_dm = firstDM;
      c_.dm_step = step;
    }
  }
  void setNrZappedChannels(unsigned int v) { c_.nr_zapped_channels = v; }

  unsigned int getNrBeams() const { return c_.nr_beams; }
  unsigned int getNrSynthesizedBeams() const { return c_.nr_synthesized_beams; }
  unsigned int getNrSamplesPerBatch(bool subbanding = false, unsigned int padding = 0) const {
    return pad(subbanding ? c_.nr_samples_per_batch_subbanding : c_.nr_samples_per_batch,
               padding);
  }
  unsigned int getNrSamplesPerDispersedBatch(bool subbanding = false,
                                             unsigned int padding = 0) const {
    return pad(subbanding ? c_.nr_samples_per_dispersed_batch_subbanding
                          : c_.nr_samples_per_dispersed_batch,
               padding);
  }
  float getSamplingTime() const { return c_.sampling_time; }
  unsigned int getDownsampling() const { return c_.downsampling; }
  unsigned int getNrChannels(unsigned int padding = 0) const { return pad(c_.nr_channels, padding); }
  unsigned int getNrSubbands(unsigned int padding = 0) const { return pad(c_.nr_subbands, padding); }
  unsigned int getNrChannelsPerSubband() const { return c_.nr_channels / c_.nr_subbands; }
  unsigned int getNrZappedChannels() const { return c_.nr_zapped_channels; }
  unsigned int getNrDMs(bool subbanding = false) const {
    return subbanding ? c_.nr_dms_subbanding : c_.nr_dms;
  }
  float getFirstDM(bool subbanding = false) const {
    return subbanding ? c_.first_dm_subbanding : c_.first_dm;
  }
  float getDMStep(bool subbanding = false) const {
    return subbanding ? c_.dm_step_subbanding : c_.dm_step;
  }
  float getMinFreq() const { return c_.min_freq; }
  float getChannelBandwidth() const { return c_.channel_bandwidth; }
  float getMaxFreq() const { return dd_max_freq(&c_); }
  float getSubbandMinFreq() const { return dd_subband_min_freq(&c_); }
  float getSubbandMaxFreq() const { return dd_subband_max_freq(&c_); }
  float getSubbandBandwidth() const { return dd_subband_bandwidth(&c_); }

  const dd_observation &c() const { return c_; }

 private:
  static unsigned int pad(unsigned int v, unsigned int p) {
    return static_cast<unsigned int>(dd_pad(v, p));
  }
  dd_observation c_;
};

}  // namespace AstroData

namespace Dedispersion {

class DedispersionError : public std::runtime_error {
 public:
  DedispersionError(int status, const std::string &what)
      : std::runtime_error(what), status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline void check(int status) {
  if (status != DD_OK) throw DedispersionError(status, dd_last_error());
}

// Dedispersion::DedispersionConf with the isa::OpenCL::KernelConf fields.
class DedispersionConf {
 public:
  DedispersionConf() { c_ = dd_conf{0, 1, 8, 32, 8, 1, 16, 4, 1}; }
  explicit DedispersionConf(const dd_conf &c) : c_(c) {}
  bool getSplitBatches() const { return c_.split_batches != 0; }
  bool getLocalMem() const { return c_.local_mem != 0; }
  unsigned int getUnroll() const { return c_.unroll; }
  void setSplitBatches(bool v) { c_.split_batches = v; }
  void setLocalMem(bool v) { c_.local_mem = v; }
  void setUnroll(unsigned int v) { c_.unroll = v; }
  unsigned int getNrThreadsD0() const { return c_.threads_d0; }
  unsigned int getNrThreadsD1() const { return c_.threads_d1; }
  unsigned int getNrThreadsD2() const { return c_.threads_d2; }
  unsigned int getNrItemsD0() const { return c_.items_d0; }
  unsigned int getNrItemsD1() const { return c_.items_d1; }
  unsigned int getNrItemsD2() const { return c_.items_d2; }
  void setNrThreadsD0(unsigned int v) { c_.threads_d0 = v; }
  void setNrThreadsD1(unsigned int v) { c_.threads_d1 = v; }
  void setNrThreadsD2(unsigned int v) { c_.threads_d2 = v; }
  void setNrItemsD0(unsigned int v) { c_.items_d0 = v; }
  void setNrItemsD1(unsigned int v) { c_.items_d1 = v; }
  void setNrItemsD2(unsigned int v) { c_.items_d2 = v; }
  // "split local unroll tD0 tD1 tD2 iD0 iD1 iD2" (src/Dedispersion.cpp:87-89)
  std::string print() const {
    char text[256];
    check(dd_conf_print(&c_, text, sizeof(text)));
    return text;
  }
  const dd_conf &c() const { return c_; }

 private:
  dd_conf c_;
};

typedef std::map<std::string, std::map<unsigned int, DedispersionConf *> *> tunedDedispersionConf;

inline std::vector<float> *getShifts(AstroData::Observation &observation,
                                     const unsigned int padding) {
  std::vector<float> *s = new std::vector<float>(observation.getNrChannels(padding / sizeof(float)));
  int st = dd_get_shifts(&observation.c(), padding, s->data(), s->size());
  if (st != DD_OK) {
    delete s;
    check(st);
  }
  return s;
}

inline std::vector<float> *getShiftsStepTwo(AstroData::Observation &observation,
                                            const unsigned int padding) {
  std::vector<float> *s = new std::vector<float>(observation.getNrSubbands(padding / sizeof(float)));
  int st = dd_get_shifts_step_two(&observation.c(), padding, s->data(), s->size());
  if (st != DD_OK) {
    delete s;
    check(st);
  }
  return s;
}

namespace detail {
template <typename I>
constexpr unsigned int storage_bits() {
  return std::is_same<I, float>::value ? 32u : static_cast<unsigned int>(sizeof(I) * 8);
}
template <typename I, typename L, typename O>
void check_types() {
  static_assert(std::is_same<L, float>::value && std::is_same<O, float>::value,
                "the engine accumulates exactly and writes float output (L = O = float)");
  static_assert(std::is_same<I, uint8_t>::value || std::is_same<I, uint16_t>::value ||
                    std::is_same<I, float>::value,
                "input type must be uint8_t (1/2/4/8 bits), uint16_t or float");
}
inline void check_size(size_t have, uint64_t need, const char *what) {
  if (have < need)
    throw DedispersionError(DD_ERR_INVALID_ARGUMENT,
                            std::string(what) + " is smaller than the reference layout needs");
}
}  // namespace detail

template <typename I, typename L, typename O>
void dedispersion(AstroData::Observation &observation, const std::vector<unsigned int> &zappedChannels,
                  const std::vector<unsigned int> &beamMapping, const std::vector<I> &input,
                  std::vector<O> &output, const std::vector<float> &shifts,
                  const unsigned int padding, const uint8_t inputBits) {
  detail::check_types<I, L, O>();
  const unsigned int bits = inputBits < 8 ? inputBits : detail::storage_bits<I>();
  dd_layout lay;
  check(dd_get_layout(&observation.c(), DD_SINGLE_STEP, bits, padding, nullptr, &lay));
  detail::check_size(input.size() * sizeof(I), lay.input_bytes, "input");
  detail::check_size(output.size() * sizeof(O), lay.output_bytes, "output");
  check(dd_dedispersion(&observation.c(), zappedChannels.data(), beamMapping.data(), input.data(),
                        output.data(), shifts.data(), padding, bits));
}

template <typename I, typename L, typename O>
void subbandDedispersionStepOne(AstroData::Observation &observation,
                                const std::vector<unsigned int> &zappedChannels,
                                const std::vector<I> &input, std::vector<O> &output,
                                const std::vector<float> &shifts, const unsigned int padding,
                                const uint8_t inputBits) {
  detail::check_types<I, L, O>();
  const unsigned int bits = inputBits < 8 ? inputBits : detail::storage_bits<I>();
  dd_layout lay;
  check(dd_get_layout(&observation.c(), DD_STEP_ONE, bits, padding, nullptr, &lay));
  detail::check_size(input.size() * sizeof(I), lay.input_bytes, "input");
  detail::check_size(output.size() * sizeof(O), lay.output_bytes, "output");
  check(dd_subband_dedispersion_step_one(&observation.c(), zappedChannels.data(), input.data(),
                                         output.data(), shifts.data(), padding, bits));
}

template <typename I, typename L, typename O>
void subbandDedispersionStepTwo(AstroData::Observation &observation,
                                const std::vector<unsigned int> &beamMapping,
                                const std::vector<I> &input, std::vector<O> &output,
                                const std::vector<float> &shifts, const unsigned int padding) {
  static_assert(std::is_same<I, float>::value, "step two reads float step-one output");
  detail::check_types<I, L, O>();
  dd_layout lay;
  check(dd_get_layout(&observation.c(), DD_STEP_TWO, 32, padding, nullptr, &lay));
  detail::check_size(input.size() * sizeof(I), lay.input_bytes, "input");
  detail::check_size(output.size() * sizeof(O), lay.output_bytes, "output");
  check(dd_subband_dedispersion_step_two(&observation.c(), beamMapping.data(), input.data(),
                                         output.data(), shifts.data(), padding));
}

// subbandDedispersionStepOne followed by subbandDedispersionStepTwo in one
// call (no reference counterpart): the intermediate stays on the device,
// packed as exact 16-bit sums of coarse-DM pairs where they fit; `output`
// equals the two calls' output bit for bit.  Input as for step one, output as
// for step two.
template <typename I, typename L, typename O>
void subbandDedispersion(AstroData::Observation &observation,
                         const std::vector<unsigned int> &zappedChannels,
                         const std::vector<unsigned int> &beamMapping, const std::vector<I> &input,
                         std::vector<O> &output, const std::vector<float> &shifts,
                         const std::vector<float> &shiftsStepTwo, const unsigned int padding,
                         const uint8_t inputBits) {
  detail::check_types<I, L, O>();
  const unsigned int bits = inputBits < 8 ? inputBits : detail::storage_bits<I>();
  dd_layout one, two;
  check(dd_get_layout(&observation.c(), DD_STEP_ONE, bits, padding, nullptr, &one));
  check(dd_get_layout(&observation.c(), DD_STEP_TWO, 32, padding, nullptr, &two));
  detail::check_size(input.size() * sizeof(I), one.input_bytes, "input");
  detail::check_size(output.size() * sizeof(O), two.output_bytes, "output");
  check(dd_subband_dedispersion(&observation.c(), zappedChannels.data(), beamMapping.data(),
                                input.data(), output.data(), shifts.data(),
                                shiftsStepTwo.data(), padding, bits));
}

// Loads every "device nrDMs split local unroll tD0 tD1 tD2 iD0 iD1 iD2"
// line; lines not starting with a letter are skipped and the first line of a
// (device, nrDMs) pair wins.  Throws AstroData::FileError if the file cannot
// be opened, DedispersionError for a malformed line.
inline void readTunedDedispersionConf(tunedDedispersionConf &tunedDedispersion,
                                      const std::string &dedispersionFilename);

}  // namespace Dedispersion

#include <cctype>
#include <fstream>
#include <sstream>

inline void Dedispersion::readTunedDedispersionConf(tunedDedispersionConf &tuned,
                                                    const std::string &filename) {
  std::ifstream in(filename);
  if (!in) throw AstroData::FileError("Impossible to open " + filename);
  std::string line;
  while (std::getline(in, line)) {
    if (line.empty() || !std::isalpha(static_cast<unsigned char>(line[0]))) continue;
    std::istringstream ls(line);
    std::string device;
    unsigned long v[10];
    ls >> device;
    for (int i = 0; i < 10; i++)
      if (!(ls >> v[i]))
        throw DedispersionError(DD_ERR_FILE, "malformed tuned-conf line in " + filename + ": " + line);
    dd_conf c{static_cast<uint32_t>(v[1] != 0), static_cast<uint32_t>(v[2] != 0),
              static_cast<uint32_t>(v[3]), static_cast<uint32_t>(v[4]),
              static_cast<uint32_t>(v[5]), static_cast<uint32_t>(v[6]),
              static_cast<uint32_t>(v[7]), static_cast<uint32_t>(v[8]),
              static_cast<uint32_t>(v[9])};
    auto it = tuned.find(device);
    if (it == tuned.end())
      it = tuned.insert(std::make_pair(device, new std::map<unsigned int, DedispersionConf *>())).first;
    if (it->second->count(static_cast<unsigned int>(v[0])) == 0)
      it->second->insert(std::make_pair(static_cast<unsigned int>(v[0]), new DedispersionConf(c)));
  }
}

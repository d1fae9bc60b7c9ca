// ref_wrapper.cpp -- C entry points around the reference's own CPU code.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile (target `ref`) into
// oracle/_ref/libddref.so from the reference's unmodified sources
// (include/Dedispersion.hpp, src/Shifts.cpp, src/Dedispersion.cpp) and the
// stand-in headers in oracle/shim/.  Used to pin the oracle restatement
// (oracle/dd_oracle.c) and to generate the golden fixtures; it never ships.
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include <Dedispersion.hpp>
#include <Shifts.hpp>

#include "../include/dedisp_gb300.h"

namespace {

AstroData::Observation to_observation(const dd_observation *o) {
  AstroData::Observation obs;
  obs.setNrBeams(o->nr_beams);
  obs.setNrSynthesizedBeams(o->nr_synthesized_beams);
  obs.setNrSamplesPerBatch(o->nr_samples_per_batch);
  obs.setNrSamplesPerBatch(o->nr_samples_per_batch_subbanding, true);
  obs.setNrSamplesPerDispersedBatch(o->nr_samples_per_dispersed_batch);
  obs.setNrSamplesPerDispersedBatch(o->nr_samples_per_dispersed_batch_subbanding, true);
  obs.setSamplingTime(o->sampling_time);
  obs.setFrequencyRange(o->nr_subbands, o->nr_channels, o->min_freq, o->channel_bandwidth);
  obs.setDMRange(o->nr_dms, o->first_dm, o->dm_step);
  obs.setDMRange(o->nr_dms_subbanding, o->first_dm_subbanding, o->dm_step_subbanding, true);
  obs.setNrZappedChannels(o->nr_zapped_channels);
  return obs;
}

template <typename T>
std::vector<T> from_ptr(const void *p, size_t n) {
  std::vector<T> v(n);
  std::memcpy(v.data(), p, n * sizeof(T));
  return v;
}

}  // namespace

extern "C" {

int ddref_get_shifts(const dd_observation *o, unsigned int padding, float *out, size_t cap) {
  AstroData::Observation obs = to_observation(o);
  std::vector<float> *s = Dedispersion::getShifts(obs, padding);
  if (s->size() > cap) { delete s; return -1; }
  std::memcpy(out, s->data(), s->size() * sizeof(float));
  int n = static_cast<int>(s->size());
  delete s;
  return n;
}

int ddref_get_shifts_step_two(const dd_observation *o, unsigned int padding, float *out, size_t cap) {
  AstroData::Observation obs = to_observation(o);
  std::vector<float> *s = Dedispersion::getShiftsStepTwo(obs, padding);
  if (s->size() > cap) { delete s; return -1; }
  std::memcpy(out, s->data(), s->size() * sizeof(float));
  int n = static_cast<int>(s->size());
  delete s;
  return n;
}

// Dedispersion::dedispersion<I, float, float>.  Element counts are the
// caller's; the vectors are exactly the reference layout.
int ddref_dedispersion(const dd_observation *o, const uint32_t *zapped, size_t n_zapped,
                       const uint32_t *mapping, size_t n_mapping, const void *input,
                       size_t n_input_elems, float *output, size_t n_output,
                       const float *shifts, size_t n_shifts, unsigned int padding,
                       unsigned int bits) {
  AstroData::Observation obs = to_observation(o);
  std::vector<unsigned int> z = from_ptr<unsigned int>(zapped, n_zapped);
  std::vector<unsigned int> m = from_ptr<unsigned int>(mapping, n_mapping);
  std::vector<float> sh = from_ptr<float>(shifts, n_shifts);
  std::vector<float> out(n_output, 0.0f);
  std::memcpy(out.data(), output, n_output * sizeof(float));
  if (bits <= 8) {
    std::vector<uint8_t> in = from_ptr<uint8_t>(input, n_input_elems);
    Dedispersion::dedispersion<uint8_t, float, float>(obs, z, m, in, out, sh, padding, static_cast<uint8_t>(bits));
  } else if (bits == 16) {
    std::vector<uint16_t> in = from_ptr<uint16_t>(input, n_input_elems);
    Dedispersion::dedispersion<uint16_t, float, float>(obs, z, m, in, out, sh, padding, static_cast<uint8_t>(bits));
  } else if (bits == 32) {
    std::vector<float> in = from_ptr<float>(input, n_input_elems);
    Dedispersion::dedispersion<float, float, float>(obs, z, m, in, out, sh, padding, static_cast<uint8_t>(bits));
  } else {
    return -1;
  }
  std::memcpy(output, out.data(), n_output * sizeof(float));
  return 0;
}

// Dedispersion::subbandDedispersionStepOne<uint8_t, float, float> (8-bit
// only: the reference's output pitch divides by 8 / inputBits).
int ddref_step_one_u8(const dd_observation *o, const uint32_t *zapped, size_t n_zapped,
                      const uint8_t *input, size_t n_input, float *output, size_t n_output,
                      const float *shifts, size_t n_shifts, unsigned int padding) {
  AstroData::Observation obs = to_observation(o);
  std::vector<unsigned int> z = from_ptr<unsigned int>(zapped, n_zapped);
  std::vector<float> sh = from_ptr<float>(shifts, n_shifts);
  std::vector<uint8_t> in = from_ptr<uint8_t>(input, n_input);
  std::vector<float> out(n_output, 0.0f);
  Dedispersion::subbandDedispersionStepOne<uint8_t, float, float>(obs, z, in, out, sh, padding, 8);
  std::memcpy(output, out.data(), n_output * sizeof(float));
  return 0;
}

// Dedispersion::subbandDedispersionStepTwo<float, float, float>.
int ddref_step_two(const dd_observation *o, const uint32_t *mapping, size_t n_mapping,
                   const float *input, size_t n_input, float *output, size_t n_output,
                   const float *shifts, size_t n_shifts, unsigned int padding) {
  AstroData::Observation obs = to_observation(o);
  std::vector<unsigned int> m = from_ptr<unsigned int>(mapping, n_mapping);
  std::vector<float> sh = from_ptr<float>(shifts, n_shifts);
  std::vector<float> in = from_ptr<float>(input, n_input);
  std::vector<float> out(n_output, 0.0f);
  Dedispersion::subbandDedispersionStepTwo<float, float, float>(obs, m, in, out, sh, padding);
  std::memcpy(output, out.data(), n_output * sizeof(float));
  return 0;
}

// Dedispersion::readTunedDedispersionConf + lookup of (device, nrDMs).
// Returns 0 on a hit, 1 if absent, -1 if the file cannot be opened.
int ddref_read_tuned_conf(const char *path, const char *device, unsigned int nr_dms,
                          dd_conf *conf, char *printed, size_t cap) {
  Dedispersion::tunedDedispersionConf db;
  try {
    Dedispersion::readTunedDedispersionConf(db, path);
  } catch (AstroData::FileError &) {
    return -1;
  }
  int rc = 1;
  auto it = db.find(device);
  if (it != db.end()) {
    auto jt = it->second->find(nr_dms);
    if (jt != it->second->end()) {
      const Dedispersion::DedispersionConf *c = jt->second;
      conf->split_batches = c->getSplitBatches();
      conf->local_mem = c->getLocalMem();
      conf->unroll = c->getUnroll();
      conf->threads_d0 = c->getNrThreadsD0();
      conf->threads_d1 = c->getNrThreadsD1();
      conf->threads_d2 = c->getNrThreadsD2();
      conf->items_d0 = c->getNrItemsD0();
      conf->items_d1 = c->getNrItemsD1();
      conf->items_d2 = c->getNrItemsD2();
      std::string p = c->print();
      std::strncpy(printed, p.c_str(), cap);
      if (cap) printed[cap - 1] = 0;
      rc = 0;
    }
  }
  for (auto &dev : db) {
    for (auto &e : *dev.second) delete e.second;
    delete dev.second;
  }
  return rc;
}

}  // extern "C"

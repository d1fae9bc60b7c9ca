// dedispersion_test.cpp -- the engine's twin of the reference's
// DedispersionTest (src/DedispersionTest.cpp): same modes and switches, same
// data generation (rand() % 10 or the constant 10; sub-byte rand() % bits or
// bits - 1), same "TEST PASSED." / "Wrong samples" report.  The device result
// comes from the drop-in C++ surface (include/dedispersion_gb300.hpp) and,
// with the tile switches, from a plan running that configuration; both are
// compared sample by sample with the CPU oracle (oracle/dd_oracle.c), the role
// the reference's CPU templates play in DedispersionTest.
//
// Test infrastructure: built and run by tests/test_cpp_surface.py.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "dedispersion_gb300.hpp"

extern "C" {
int ddo_dedispersion(const dd_observation *, const uint32_t *, const uint32_t *, const void *,
                     float *, const float *, uint32_t, uint32_t, uint32_t, uint32_t, int);
int ddo_step_one(const dd_observation *, const uint32_t *, const void *, float *, const float *,
                 uint32_t, uint32_t, int);
int ddo_step_two(const dd_observation *, const uint32_t *, const float *, float *, const float *,
                 uint32_t, int);
}

namespace {

struct Args {
  int argc;
  char **argv;
  bool has(const char *s) const {
    for (int i = 1; i < argc; i++)
      if (!std::strcmp(argv[i], s)) return true;
    return false;
  }
  std::string get(const char *s) const {
    for (int i = 1; i + 1 < argc; i++)
      if (!std::strcmp(argv[i], s)) return argv[i + 1];
    throw std::runtime_error(std::string("missing switch ") + s);
  }
  template <typename T>
  T num(const char *s) const {
    return static_cast<T>(std::stod(get(s)));
  }
  template <typename T>
  T num(const char *s, T def) const {
    return has(s) ? num<T>(s) : def;
  }
};

// AstroData::readZappedChannels: whitespace-separated channel indices.
void read_zapped(const std::string &path, std::vector<unsigned int> &zapped) {
  std::ifstream in(path);
  if (!in) throw AstroData::FileError("Impossible to open " + path);
  long c;
  while (in >> c)
    if (c >= 0 && static_cast<size_t>(c) < zapped.size()) zapped[c] = 1;
}

void put_subbyte(std::vector<uint8_t> &buf, size_t row, size_t k, unsigned bits, unsigned v) {
  const unsigned per = 8 / bits;
  uint8_t &b = buf[row + k / per];
  const unsigned first = (k % per) * bits;
  b = static_cast<uint8_t>((b & ~(((1u << bits) - 1u) << first)) | (v << first));
}

}  // namespace

int main(int argc, char **argv) {
  Args a{argc, argv};
  const bool single = a.has("-single_step"), one = a.has("-step_one"), two = a.has("-step_two");
  if (single + one + two != 1) {
    std::cerr << "Mutually exclusive modes, select one: -single_step -step_one -step_two" << std::endl;
    return 1;
  }
  const bool random = a.has("-random");
  unsigned padding = 0, bits = 8;
  Dedispersion::DedispersionConf conf;
  AstroData::Observation obs;
  std::string zfile;
  try {
    padding = a.num<unsigned>("-padding");
    bits = a.num<unsigned>("-input_bits", 8u);
    srand(a.num<unsigned>("-seed", 1u));
    if (a.has("-threadsD0")) {
      conf.setNrThreadsD0(a.num<unsigned>("-threadsD0"));
      conf.setNrThreadsD1(a.num<unsigned>("-threadsD1"));
      conf.setNrItemsD0(a.num<unsigned>("-itemsD0"));
      conf.setNrItemsD1(a.num<unsigned>("-itemsD1"));
      conf.setUnroll(a.num<unsigned>("-unroll"));
      conf.setLocalMem(true);
    }
    obs.setNrBeams(a.num<unsigned>("-beams"));
    obs.setNrSamplesPerBatch(a.num<unsigned>("-samples"));
    obs.setSamplingTime(a.num<float>("-sampling_time"));
    if (single || one) zfile = a.get("-zapped_channels");
    if (single) {
      obs.setNrSynthesizedBeams(a.num<unsigned>("-synthesized_beams"));
      obs.setFrequencyRange(1, a.num<unsigned>("-channels"), a.num<float>("-min_freq"),
                            a.num<float>("-channel_bandwidth"));
      obs.setDMRange(a.num<unsigned>("-dms"), a.num<float>("-dm_first"), a.num<float>("-dm_step"));
    } else if (one) {
      obs.setFrequencyRange(a.num<unsigned>("-subbands"), a.num<unsigned>("-channels"),
                            a.num<float>("-min_freq"), a.num<float>("-channel_bandwidth"));
      obs.setDMRange(a.num<unsigned>("-subbanding_dms"), a.num<float>("-subbanding_dm_first"),
                     a.num<float>("-subbanding_dm_step"), true);
      obs.setDMRange(a.num<unsigned>("-dms"), a.num<float>("-dm_first"), a.num<float>("-dm_step"));
    } else {
      obs.setNrSynthesizedBeams(a.num<unsigned>("-synthesized_beams"));
      obs.setFrequencyRange(a.num<unsigned>("-subbands"), a.num<unsigned>("-channels"),
                            a.num<float>("-min_freq"), a.num<float>("-channel_bandwidth"));
      obs.setDMRange(a.num<unsigned>("-subbanding_dms"), 0.0f, 0.0f, true);
      obs.setDMRange(a.num<unsigned>("-dms"), a.num<float>("-dm_first"), a.num<float>("-dm_step"));
    }
  } catch (std::exception &e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }

  std::vector<float> *shifts = Dedispersion::getShifts(obs, padding);
  std::vector<float> *shifts2 = Dedispersion::getShiftsStepTwo(obs, padding);
  std::vector<unsigned int> zapped(obs.getNrChannels(padding / sizeof(unsigned int)));
  std::vector<unsigned int> mapping;
  if (single || one) read_zapped(zfile, zapped);
  // Dispersed lengths as src/DedispersionTest.cpp:129, 145-146 set them.
  if (single) {
    obs.setNrSamplesPerDispersedBatch(static_cast<unsigned>(std::ceil(
        obs.getNrSamplesPerBatch() +
        (shifts->at(0) * (obs.getFirstDM() + ((obs.getNrDMs() - 1) * obs.getDMStep()))))));
  } else {
    obs.setNrSamplesPerBatch(static_cast<unsigned>(std::ceil(
        obs.getNrSamplesPerBatch() +
        (shifts2->at(0) * (obs.getFirstDM() + ((obs.getNrDMs() - 1) * obs.getDMStep()))))), true);
    if (one)
      obs.setNrSamplesPerDispersedBatch(static_cast<unsigned>(std::ceil(
          obs.getNrSamplesPerBatch(true) +
          (shifts->at(0) * (obs.getFirstDM(true) + ((obs.getNrDMs(true) - 1) * obs.getDMStep(true)))))),
          true);
  }
  const dd_mode mode = single ? DD_SINGLE_STEP : (one ? DD_STEP_ONE : DD_STEP_TWO);
  dd_layout lay;
  Dedispersion::check(dd_get_layout(&obs.c(), mode, two ? 32 : bits, padding, nullptr, &lay));
  std::vector<float> out(lay.output_bytes / 4, 0.0f), out_c(lay.output_bytes / 4, 0.0f),
      out_plan(lay.output_bytes / 4, 0.0f);
  std::vector<uint8_t> in8;
  std::vector<float> inf;
  const size_t rows = two ? (size_t)obs.getNrBeams() * obs.getNrDMs(true) * obs.getNrSubbands()
                          : (size_t)obs.getNrBeams() * obs.getNrChannels();
  const unsigned samples = single ? obs.getNrSamplesPerDispersedBatch()
                                  : (one ? obs.getNrSamplesPerDispersedBatch(true)
                                         : obs.getNrSamplesPerBatch(true));
  if (two) {
    inf.assign(lay.input_bytes / 4, 0.0f);
    for (size_t r = 0; r < rows; r++)
      for (unsigned s = 0; s < samples; s++)
        inf[r * (lay.input_row_bytes / 4) + s] = random ? static_cast<float>(rand() % 10) : 10.0f;
    mapping.assign((size_t)obs.getNrSynthesizedBeams() * lay.mapping_row_elems, 0);
    for (unsigned b = 0; b < obs.getNrSynthesizedBeams(); b++)
      for (unsigned s = 0; s < obs.getNrSubbands(); s++)
        mapping[b * lay.mapping_row_elems + s] = b % obs.getNrBeams();
  } else {
    in8.assign(lay.input_bytes, 0);
    for (size_t r = 0; r < rows; r++)
      for (unsigned s = 0; s < samples; s++) {
        if (bits >= 8)
          in8[r * lay.input_row_bytes + s] = static_cast<uint8_t>(random ? rand() % 10 : 10);
        else
          put_subbyte(in8, r * lay.input_row_bytes, s, bits,
                      random ? static_cast<unsigned>(rand()) % bits : bits - 1);
      }
    if (single) {
      mapping.assign((size_t)obs.getNrSynthesizedBeams() * lay.mapping_row_elems, 0);
      for (unsigned b = 0; b < obs.getNrSynthesizedBeams(); b++)
        for (unsigned c = 0; c < obs.getNrChannels(); c++)
          mapping[b * lay.mapping_row_elems + c] = b % obs.getNrBeams();
    }
  }

  try {
    // The drop-in path.
    if (single)
      Dedispersion::dedispersion<uint8_t, float, float>(obs, zapped, mapping, in8, out, *shifts,
                                                        padding, static_cast<uint8_t>(bits));
    else if (one)
      Dedispersion::subbandDedispersionStepOne<uint8_t, float, float>(
          obs, zapped, in8, out, *shifts, padding, static_cast<uint8_t>(bits));
    else
      Dedispersion::subbandDedispersionStepTwo<float, float, float>(obs, mapping, inf, out,
                                                                    *shifts2, padding);
    // The plan path with the requested tile configuration.
    dd_plan *plan = nullptr;
    Dedispersion::check(dd_plan_create(&plan, &obs.c(), mode, two ? 32 : bits, padding,
                                       a.has("-threadsD0") ? &conf.c() : nullptr, 0));
    Dedispersion::check(dd_plan_set_shifts(plan, two ? shifts2->data() : shifts->data(),
                                           two ? shifts2->size() : shifts->size()));
    if (!two) Dedispersion::check(dd_plan_set_zapped(plan, zapped.data(), zapped.size()));
    if (!one) Dedispersion::check(dd_plan_set_beam_mapping(plan, mapping.data(), mapping.size()));
    void *d_in = nullptr;
    float *d_out = nullptr;
    if (cudaMalloc(&d_in, lay.input_bytes) != cudaSuccess ||
        cudaMalloc(&d_out, lay.output_bytes) != cudaSuccess)
      throw std::runtime_error("cudaMalloc failed");
    cudaMemcpy(d_in, two ? static_cast<const void *>(inf.data()) : in8.data(), lay.input_bytes,
               cudaMemcpyHostToDevice);
    cudaMemset(d_out, 0, lay.output_bytes);
    Dedispersion::check(dd_plan_run(plan, d_in, d_out, nullptr));
    Dedispersion::check(dd_plan_check(plan, nullptr));
    cudaMemcpy(out_plan.data(), d_out, lay.output_bytes, cudaMemcpyDeviceToHost);
    cudaFree(d_in);
    cudaFree(d_out);
    dd_plan_destroy(plan);
  } catch (std::exception &e) {
    std::cerr << "GPU path error: " << e.what() << std::endl;
    return 1;
  }

  int rc;
  if (single)
    rc = ddo_dedispersion(&obs.c(), zapped.data(), mapping.data(), in8.data(), out_c.data(),
                          shifts->data(), padding, bits, 0, 0, 4);
  else if (one)
    rc = ddo_step_one(&obs.c(), zapped.data(), in8.data(), out_c.data(), shifts->data(), padding,
                      bits, 4);
  else
    rc = ddo_step_two(&obs.c(), mapping.data(), inf.data(), out_c.data(), shifts2->data(),
                      padding, 4);
  if (rc != 0) {
    std::cerr << "oracle failed" << std::endl;
    return 1;
  }

  const size_t out_rows = lay.output_bytes / 4 / lay.output_row_elems;
  const unsigned valid = single || two ? obs.getNrSamplesPerBatch() : obs.getNrSamplesPerBatch(true);
  uint64_t wrong = 0;
  for (size_t r = 0; r < out_rows; r++)
    for (unsigned s = 0; s < valid; s++) {
      const size_t i = r * lay.output_row_elems + s;
      if (std::memcmp(&out[i], &out_c[i], 4) != 0 || std::memcmp(&out_plan[i], &out_c[i], 4) != 0)
        wrong++;
    }
  if (wrong > 0)
    std::cout << "Wrong samples: " << wrong << " (" << (wrong * 100.0) / (double)(out_rows * valid)
              << "%)." << std::endl;
  else
    std::cout << "TEST PASSED." << std::endl;
  delete shifts;
  delete shifts2;
  return wrong > 0 ? 2 : 0;
}

// subband_test.cpp -- the C++ surface's one-call subband method
// (Dedispersion::subbandDedispersion in include/dedispersion_gb300.hpp)
// against the CPU oracle's step one followed by its step two
// (oracle/dd_oracle.c), sample by sample.  Geometry as the reference's test
// driver derives it for the two steps (src/DedispersionTest.cpp:145-146).
//
// Usage: subband_test <channels> <subbands> <coarse DMs> <fine DMs> <bits>
//        <beams> <synthesized beams> <seed>
// Test infrastructure: built and run by tests/test_cpp_surface.py.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <vector>

#include "dedispersion_gb300.hpp"

extern "C" {
int ddo_step_one(const dd_observation *, const uint32_t *, const void *, float *, const float *,
                 uint32_t, uint32_t, int);
int ddo_step_two(const dd_observation *, const uint32_t *, const float *, float *, const float *,
                 uint32_t, int);
}

int main(int argc, char **argv) {
  if (argc != 9) {
    std::cerr << "usage: subband_test C SB D1 D2 bits beams sbeams seed" << std::endl;
    return 1;
  }
  const unsigned C = std::atoi(argv[1]), SB = std::atoi(argv[2]), D1 = std::atoi(argv[3]);
  const unsigned D2 = std::atoi(argv[4]), bits = std::atoi(argv[5]);
  const unsigned beams = std::atoi(argv[6]), sbeams = std::atoi(argv[7]);
  srand(std::atoi(argv[8]));
  const unsigned padding = 128;
  AstroData::Observation obs;
  obs.setNrBeams(beams);
  obs.setNrSynthesizedBeams(sbeams);
  obs.setNrSamplesPerBatch(2048);
  obs.setSamplingTime(0.00008192f);
  obs.setFrequencyRange(SB, C, 1220.0f, 0.1953125f);
  obs.setDMRange(D1, 0.0f, 3.2f, true);
  obs.setDMRange(D2, 0.0f, 0.2f);
  std::vector<float> *shifts = Dedispersion::getShifts(obs, padding);
  std::vector<float> *shifts2 = Dedispersion::getShiftsStepTwo(obs, padding);
  obs.setNrSamplesPerBatch(static_cast<unsigned>(std::ceil(
      obs.getNrSamplesPerBatch() +
      (shifts2->at(0) * (obs.getFirstDM() + ((obs.getNrDMs() - 1) * obs.getDMStep()))))), true);
  obs.setNrSamplesPerDispersedBatch(static_cast<unsigned>(std::ceil(
      obs.getNrSamplesPerBatch(true) +
      (shifts->at(0) * (obs.getFirstDM(true) + ((obs.getNrDMs(true) - 1) * obs.getDMStep(true)))))),
      true);
  dd_layout one, two;
  Dedispersion::check(dd_get_layout(&obs.c(), DD_STEP_ONE, bits, padding, nullptr, &one));
  Dedispersion::check(dd_get_layout(&obs.c(), DD_STEP_TWO, 32, padding, nullptr, &two));
  std::vector<unsigned int> zapped(obs.getNrChannels(padding / sizeof(unsigned int)), 0);
  for (unsigned c = 3; c < C; c += 29) zapped[c] = 1;
  std::vector<unsigned int> mapping((size_t)sbeams * two.mapping_row_elems, 0);
  for (unsigned b = 0; b < sbeams; b++)
    for (unsigned s = 0; s < SB; s++) mapping[b * two.mapping_row_elems + s] = (b + s) % beams;
  std::vector<uint8_t> in(one.input_bytes);
  for (auto &v : in) v = static_cast<uint8_t>(rand());
  std::vector<float> out(two.output_bytes / 4, 0.0f), mid(one.output_bytes / 4, 0.0f),
      want(two.output_bytes / 4, 0.0f);
  try {
    Dedispersion::subbandDedispersion<uint8_t, float, float>(obs, zapped, mapping, in, out,
                                                             *shifts, *shifts2, padding,
                                                             static_cast<uint8_t>(bits));
  } catch (std::exception &e) {
    std::cerr << "GPU path error: " << e.what() << std::endl;
    return 1;
  }
  if (ddo_step_one(&obs.c(), zapped.data(), in.data(), mid.data(), shifts->data(), padding, bits,
                   4) ||
      ddo_step_two(&obs.c(), mapping.data(), mid.data(), want.data(), shifts2->data(), padding,
                   4)) {
    std::cerr << "oracle failed" << std::endl;
    return 1;
  }
  const unsigned S = obs.getNrSamplesPerBatch();
  const size_t rows = (size_t)sbeams * D1 * D2;
  size_t wrong = 0;
  for (size_t r = 0; r < rows; r++)
    for (unsigned t = 0; t < S; t++)
      if (out[r * two.output_row_elems + t] != want[r * two.output_row_elems + t]) wrong++;
  delete shifts;
  delete shifts2;
  if (wrong) {
    std::cout << "Wrong samples: " << wrong << " (" << 100.0 * wrong / (rows * S) << "%)."
              << std::endl;
    return 1;
  }
  std::cout << "TEST PASSED." << std::endl;
  return 0;
}

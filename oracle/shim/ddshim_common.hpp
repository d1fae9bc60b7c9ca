// ddshim_common.hpp -- stand-ins for the external names that the
// reference's sources use (AstroData::Observation, isa::utils, isa::OpenCL).
//
// TEST INFRASTRUCTURE ONLY: these headers exist so that the reference's own
// CPU templates (include/Dedispersion.hpp:70-176), getShifts
// (src/Shifts.cpp) and readTunedDedispersionConf (src/Dedispersion.cpp)
// compile unmodified with g++ into oracle/_ref/.  Each declaration provides
// only what those files use, written from how they use it.  AstroData and
// isa::* are not part of the reference tree; where their semantics matter
// (frequency getters, pad) the choice is stated beside the code and is the
// same one the oracle restatement and the shipped library make.
#pragma once

#include <cmath>
#include <cstdint>
#include <sstream>
#include <stdexcept>
#include <string>

namespace isa {
namespace utils {

// Round `value` up to a multiple of `padding`; padding 0 leaves it alone.
template <typename T>
inline T pad(T value, T padding) {
  if (padding == 0) return value;
  return ((value + padding - 1) / padding) * padding;
}
inline unsigned int pad(unsigned int value, unsigned long padding) {
  return pad<unsigned long>(value, padding);
}

// Bit `pos` of `value` (0 or 1).
template <typename T>
inline T getBit(T value, unsigned int pos) {
  return static_cast<T>((static_cast<unsigned long long>(value) >> pos) & 1ull);
}

// Set bit `pos` of `value` to `bit` (0 or 1).
template <typename T, typename B>
inline void setBit(T &value, B bit, unsigned int pos) {
  unsigned long long v = static_cast<unsigned long long>(static_cast<typename std::make_unsigned<T>::type>(value));
  if (bit) v |= (1ull << pos); else v &= ~(1ull << pos);
  value = static_cast<T>(v);
}

// Parse a string as T with stream extraction ("1"/"0" for bool).
template <typename S, typename T>
inline T castToType(const S &text) {
  std::istringstream in(text);
  T value{};
  in >> value;
  return value;
}

// Replace every occurrence of `placeholder` in `*src`; optionally delete src.
inline std::string *replace(std::string *src, const std::string &placeholder,
                            const std::string &value, bool deleteSrc = false) {
  std::string *out = new std::string(*src);
  std::string::size_type pos = 0;
  while ((pos = out->find(placeholder, pos)) != std::string::npos) {
    out->replace(pos, placeholder.size(), value);
    pos += value.size();
  }
  if (deleteSrc) delete src;
  return out;
}

}  // namespace utils

namespace OpenCL {

// Launch geometry of a generated kernel: threads and items per dimension.
class KernelConf {
 public:
  KernelConf() : nrThreadsD0(1), nrThreadsD1(1), nrThreadsD2(1), nrItemsD0(1), nrItemsD1(1), nrItemsD2(1) {}
  unsigned int getNrThreadsD0() const { return nrThreadsD0; }
  unsigned int getNrThreadsD1() const { return nrThreadsD1; }
  unsigned int getNrThreadsD2() const { return nrThreadsD2; }
  unsigned int getNrItemsD0() const { return nrItemsD0; }
  unsigned int getNrItemsD1() const { return nrItemsD1; }
  unsigned int getNrItemsD2() const { return nrItemsD2; }
  void setNrThreadsD0(unsigned int v) { nrThreadsD0 = v; }
  void setNrThreadsD1(unsigned int v) { nrThreadsD1 = v; }
  void setNrThreadsD2(unsigned int v) { nrThreadsD2 = v; }
  void setNrItemsD0(unsigned int v) { nrItemsD0 = v; }
  void setNrItemsD1(unsigned int v) { nrItemsD1 = v; }
  void setNrItemsD2(unsigned int v) { nrItemsD2 = v; }
  // "tD0 tD1 tD2 iD0 iD1 iD2", the column order of a tuned-conf line
  // after "split local unroll" (src/Dedispersion.cpp:32-69).
  std::string print() const {
    return std::to_string(nrThreadsD0) + " " + std::to_string(nrThreadsD1) + " " +
           std::to_string(nrThreadsD2) + " " + std::to_string(nrItemsD0) + " " +
           std::to_string(nrItemsD1) + " " + std::to_string(nrItemsD2);
  }

 private:
  unsigned int nrThreadsD0, nrThreadsD1, nrThreadsD2;
  unsigned int nrItemsD0, nrItemsD1, nrItemsD2;
};

// OpenCL C source text of bit access, used only by the string generators.
inline std::string getBit(const std::string &value, const std::string &bit) {
  return "((" + value + " >> (" + bit + ")) & 1)";
}
inline std::string setBit(const std::string &value, const std::string &bit,
                          const std::string &pos) {
  return value + " = (" + value + " & ~(1 << (" + pos + "))) | ((" + bit + ") << (" + pos + "));\n";
}

}  // namespace OpenCL
}  // namespace isa

namespace AstroData {

class FileError : public std::runtime_error {
 public:
  explicit FileError(const std::string &what) : std::runtime_error(what) {}
};

// Observation geometry.  Frequencies: maxFreq = minFreq + (C - 1) * bw; the
// subband frequency of a subband is that of its highest channel.
class Observation {
 public:
  void setNrBeams(unsigned int v) { nrBeams = v; }
  void setNrSynthesizedBeams(unsigned int v) { nrSynthesizedBeams = v; }
  void setNrSamplesPerBatch(unsigned int v, bool subbanding = false) {
    (subbanding ? nrSamplesPerBatchSubbanding : nrSamplesPerBatch) = v;
  }
  void setNrSamplesPerDispersedBatch(unsigned int v, bool subbanding = false) {
    (subbanding ? nrSamplesPerDispersedBatchSubbanding : nrSamplesPerDispersedBatch) = v;
  }
  void setSamplingTime(float v) { samplingTime = v; }
  void setFrequencyRange(unsigned int subbands, unsigned int channels, float minF, float bw) {
    nrSubbands = subbands;
    nrChannels = channels;
    minFreq = minF;
    channelBandwidth = bw;
  }
  void setDMRange(unsigned int n, float first, float step, bool subbanding = false) {
    if (subbanding) { nrDMsSubbanding = n; firstDMSubbanding = first; dmStepSubbanding = step; }
    else { nrDMs = n; firstDM = first; dmStep = step; }
  }
  void setNrZappedChannels(unsigned int v) { nrZappedChannels = v; }

  unsigned int getNrBeams() const { return nrBeams; }
  unsigned int getNrSynthesizedBeams() const { return nrSynthesizedBeams; }
  unsigned int getNrSamplesPerBatch(bool subbanding = false, unsigned int padding = 0) const {
    return isa::utils::pad(subbanding ? nrSamplesPerBatchSubbanding : nrSamplesPerBatch, padding);
  }
  unsigned int getNrSamplesPerDispersedBatch(bool subbanding = false, unsigned int padding = 0) const {
    return isa::utils::pad(subbanding ? nrSamplesPerDispersedBatchSubbanding : nrSamplesPerDispersedBatch, padding);
  }
  float getSamplingTime() const { return samplingTime; }
  unsigned int getDownsampling() const { return 1; }
  unsigned int getNrChannels(unsigned int padding = 0) const { return isa::utils::pad(nrChannels, padding); }
  unsigned int getNrSubbands(unsigned int padding = 0) const { return isa::utils::pad(nrSubbands, padding); }
  unsigned int getNrChannelsPerSubband() const { return nrChannels / nrSubbands; }
  unsigned int getNrZappedChannels() const { return nrZappedChannels; }
  unsigned int getNrDMs(bool subbanding = false) const { return subbanding ? nrDMsSubbanding : nrDMs; }
  float getFirstDM(bool subbanding = false) const { return subbanding ? firstDMSubbanding : firstDM; }
  float getDMStep(bool subbanding = false) const { return subbanding ? dmStepSubbanding : dmStep; }
  float getMinFreq() const { return minFreq; }
  float getChannelBandwidth() const { return channelBandwidth; }
  float getMaxFreq() const { return minFreq + ((nrChannels - 1) * channelBandwidth); }
  float getSubbandBandwidth() const { return (nrChannels / nrSubbands) * channelBandwidth; }
  float getSubbandMinFreq() const { return minFreq + (((nrChannels / nrSubbands) - 1) * channelBandwidth); }
  float getSubbandMaxFreq() const { return getSubbandMinFreq() + ((nrSubbands - 1) * getSubbandBandwidth()); }

 private:
  unsigned int nrBeams = 1, nrSynthesizedBeams = 1;
  unsigned int nrSamplesPerBatch = 0, nrSamplesPerBatchSubbanding = 0;
  unsigned int nrSamplesPerDispersedBatch = 0, nrSamplesPerDispersedBatchSubbanding = 0;
  float samplingTime = 0.0f;
  unsigned int nrSubbands = 1, nrChannels = 0, nrZappedChannels = 0;
  float minFreq = 0.0f, channelBandwidth = 0.0f;
  unsigned int nrDMs = 0, nrDMsSubbanding = 0;
  float firstDM = 0.0f, dmStep = 0.0f, firstDMSubbanding = 0.0f, dmStepSubbanding = 0.0f;
};

}  // namespace AstroData

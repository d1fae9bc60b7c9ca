// dd_tmem.cuh -- the TMEM-window tile (kFamilyTmem32) for float32 input in
// single-step form.
//
// The scalar float tile issues one shared-memory load per add, so the
// shared-memory port (32 words per SM clock against 128 float adds) bounds
// it at a quarter of the add rate.  This tile keeps each thread's window of
// input samples in tensor memory (TMEM, 128 lanes x 512 columns of 32 bits
// per SM), whose loads run at a warp-uniform column address:
//
//   * warp w uses TMEM lanes 32 (w % 4) .. + 31 (lane quarter q = w % 4);
//     lane l of quarter q owns output samples t0 + 16 l .. + 15;
//   * quarter q computes DMs d0 + 16 q .. + 15, its four warps four DMs each
//     (tile: 512 samples x 64 DMs);
//   * a row's window for quarter q starts at W_q = t0 + delay(row, d0 + 16 q)
//     rounded down to 4 samples; lane l holds window samples 16 l .. 16 l + 63
//     in 64 columns, so DM d's 16 samples are the 16 columns from
//     o = t0 + delay(row, d) - W_q (<= 48, checked on the host);
//   * one tcgen05.ld of 16 columns feeds 16 float adds.
//
// Rows are summed in the reference's channel order (include/Dedispersion.hpp:
// 79-104), so results equal the scalar tile's bit for bit.
//
// Per step of 4 rows: 16-byte asynchronous copies stage each row's window
// (768 floats from W_0, one pad chunk per 8 so that the lanes' 16-byte loads
// at a 64-byte stride spread over the banks) into one of 3 slots; every warp
// copies 16 of its quarter's 64 columns into TMEM (tcgen05.st; only the
// columns the row's DMs reach); after a block barrier the warps add from
// TMEM while the next rows' copies are in flight.  Two TMEM buffers of 4
// rows x 64 columns alternate between steps (all 512 columns, one CTA per
// SM).  Every wait for a copy is bounded as in the other families; a wait
// that runs out sets kStatusTimeout, lets the copies in flight land, frees
// the TMEM and returns.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>

#include "dd_internal.h"

namespace dd {

constexpr int kTmThreads = 512;
constexpr int kTmT = 16;                    // samples per lane
constexpr int kTmTileT = 32 * kTmT;         // 512 samples per tile
constexpr int kTmDPW = 4;                   // DMs per warp
constexpr int kTmTileD = 64;                // DMs per tile (16 per quarter)
constexpr int kTmRows = 4;                  // rows per step
constexpr uint32_t kTmCols = 64;            // TMEM columns per row window
constexpr uint32_t kTmMaxOff = kTmCols - kTmT;  // 48
constexpr uint32_t kTmChunks = 192;         // 16-byte chunks of a staged window
constexpr uint32_t kTmMaxQuarterOff = kTmChunks - 4 * 31 - 16;  // 52 chunks
constexpr uint32_t kTmRowBytes = (kTmChunks + kTmChunks / 8) * 16;  // 3456
constexpr uint32_t kTmSlots = 3;
constexpr uint32_t kTmSlotBytes = kTmRows * kTmRowBytes;
constexpr uint32_t kTmTabWords = 32;  // per row: rel, row, off[4], cols[4], 16 DM offset words

// Dynamic shared memory of a launch whose groups have at most `rows` rows:
// the staging slots, then each row's delay per unit DM and 16-byte chunk
// index.
__host__ __device__ inline size_t tmem_smem_bytes(uint32_t rows) {
  return (size_t)kTmSlots * kTmSlotBytes + 8u * (size_t)rows;
}

// Whether every row's windows fit the tile: within each quarter's 16 DMs the
// offset o stays <= 48, and each quarter's window start stays within 52
// chunks of the row's staged window.  Host and device round alike
// (host_delay / dev_delay).
inline bool tmem_fits(const float *shifts, size_t n, float first_dm, float dm_step,
                      uint32_t nr_dms) {
  if (nr_dms == 0) return true;
  const uint32_t tiles = (nr_dms + kTmTileD - 1) / kTmTileD;
  for (size_t i = 0; i < n; i++)
    for (uint32_t t = 0; t < tiles; t++) {
      const uint32_t d0 = t * kTmTileD;
      const uint32_t w0 = host_delay(first_dm, dm_step, d0, shifts[i]) & ~3u;
      for (uint32_t q = 0; q < 4; q++) {
        const uint32_t dq = std::min(d0 + 16u * q, nr_dms - 1);
        const uint32_t dl = std::min(d0 + 16u * q + 15u, nr_dms - 1);
        const uint32_t wq = host_delay(first_dm, dm_step, dq, shifts[i]) & ~3u;
        if (host_delay(first_dm, dm_step, dl, shifts[i]) - wq > kTmMaxOff) return false;
        if ((wq - w0) / 4u > kTmMaxQuarterOff) return false;
      }
    }
  return true;
}

}  // namespace dd

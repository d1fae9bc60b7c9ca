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
// at a 64-byte stride spread over the banks) and its offset entry (built on
// the host by tmem_tables: W_q - W_0, the columns to stage and every DM's o)
// into one of 3 slots; every warp
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
#include <vector>

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

constexpr uint32_t kTmTabWords = 20;  // per (DM tile, delay row): see tmem_tables
constexpr uint32_t kTmTabChunks = kTmTabWords / 4;

// Dynamic shared memory of a launch whose groups have at most `rows` rows:
// the staging slots, then each row's delay per unit DM, 16-byte chunk index
// and delay-table row.
__host__ __device__ inline size_t tmem_smem_bytes(uint32_t rows) {
  return (size_t)kTmSlots * kTmSlotBytes + 12u * (size_t)rows;
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

// The tile's offsets of every (DM tile, delay row), 20 words each, so that
// the kernel fetches them with the row instead of evaluating delays: word 0
// the delay of the tile's first DM rounded down to 4 samples (B), word 1
// byte q each quarter's window start (W_q - B) / 4 in chunks, word 2 byte q
// the TMEM columns quarter q stages (a multiple of 8), word 4 + 4q + k
// bytes j the offset o of DM 16q + 4k + j.  Time tiles start at multiples of
// 512 samples, so none of these depends on the time tile.  Host delays round
// as the device's (host_delay).
inline void tmem_tables(const std::vector<float> &row_shift, float first_dm, float dm_step,
                        uint32_t nr_dms, std::vector<uint32_t> *out) {
  const uint32_t tiles = nr_dms ? (nr_dms + kTmTileD - 1) / kTmTileD : 0;
  const size_t rows = row_shift.size();
  out->assign((size_t)tiles * rows * kTmTabWords, 0u);
  for (uint32_t t = 0; t < tiles; t++)
    for (size_t r = 0; r < rows; r++) {
      const float sh = row_shift[r];
      uint32_t *e = out->data() + ((size_t)t * rows + r) * kTmTabWords;
      const uint32_t d0 = t * kTmTileD, last = nr_dms - 1;
      const uint32_t b = host_delay(first_dm, dm_step, d0, sh) & ~3u;
      e[0] = b;
      for (uint32_t q = 0; q < 4; q++) {
        const uint32_t wq = host_delay(first_dm, dm_step, std::min(d0 + 16u * q, last), sh) & ~3u;
        uint32_t omax = 0;
        for (uint32_t j = 0; j < 16; j++) {
          const uint32_t d = std::min(d0 + 16u * q + j, last);
          const uint32_t o = std::min(host_delay(first_dm, dm_step, d, sh) - wq, kTmMaxOff);
          omax = std::max(omax, o);
          e[4 + 4 * q + j / 4] |= o << (8 * (j % 4));
        }
        e[1] |= std::min((wq - b) / 4u, kTmMaxQuarterOff) << (8 * q);
        e[2] |= ((omax + kTmT + 7u) & ~7u) << (8 * q);
      }
    }
}

}  // namespace dd

// shared_tables_test.cu -- host check of the shared-partial-sum stage
// tables: a CPU replay of the kernel's indexing (dd_shared.cuh) over the
// tables build_shared_tables makes, against the direct sum.
//
//   shared_tables_test <shifts.f32> <rows> <dms> <samples> <first_dm>
//                      <dm_step> <nw> <nd> <ty> <seed> <time_tiles> [smem]
//
// Checks, for every DM tile and the first <time_tiles> time tiles: every
// shared-memory read and write stays in its buffer, phase B reads only words
// phase A wrote (or the zero series), no 16-bit lane leaves its range, and
// every output sample equals the direct sum.  Prints "PASS ..." or the first
// failure.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "../../dedispersion_gb300/csrc/dd_shared_plan.h"
#include "../../dedispersion_gb300/csrc/dd_shared.cuh"

using namespace dd;

static int fail(const char *what, long a, long b, long c) {
  printf("FAIL %s %ld %ld %ld\n", what, a, b, c);
  return 1;
}

static uint32_t prmt4140(uint32_t w) { return (w & 0xFF) | ((w >> 8 & 0xFF) << 16); }
static uint32_t prmt4342(uint32_t w) { return (w >> 16 & 0xFF) | ((w >> 24) << 16); }

int main(int argc, char **argv) {
  if (argc != 12 && argc != 13) {
    fprintf(stderr, "usage: see header\n");
    return 2;
  }
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  const uint32_t K = (uint32_t)atoi(argv[2]), D = (uint32_t)atoi(argv[3]);
  const uint32_t S = (uint32_t)atoi(argv[4]);
  const float first = (float)atof(argv[5]), step = (float)atof(argv[6]);
  const int NW = atoi(argv[7]), ND = atoi(argv[8]), TY = atoi(argv[9]);
  const unsigned seed = (unsigned)atoi(argv[10]);
  const uint32_t ntt = (uint32_t)atoi(argv[11]);
  const size_t budget = argc == 13 ? (size_t)atol(argv[12]) : 232448;
  std::vector<float> shift(K);
  if (fread(shift.data(), sizeof(float), K, f) != K) return 2;
  fclose(f);

  KernelInfo k{};
  k.name = "emulated";
  k.family = kFamilyShared8;
  k.elem_bits = 8;
  k.tile_t = 64 * NW;
  k.tile_d = TY * ND;
  k.threads = 32 * TY;
  k.channels = kSharedRows;
  SharedTables tab;
  const std::string why = build_shared_tables(k, shift, first, step, D, 8, budget, &tab);
  if (!why.empty()) {
    printf("UNSUPPORTED %s\n", why.c_str());
    return 3;
  }
  if (tab.smem > budget) return fail("smem over budget", (long)tab.smem, (long)budget, 0);
  const uint32_t T = k.tile_t, DB = k.tile_d;
  const uint32_t tiles_d = (D + DB - 1) / DB;
  const uint32_t tiles_t = (S + T - 1) / T;
  uint32_t maxdelay = 0;
  for (uint32_t r = 0; r < K; r++) maxdelay = std::max(maxdelay, host_delay(first, step, D - 1, shift[r]));
  const uint32_t rowlen = (S + maxdelay + 127) / 128 * 128;
  std::mt19937 rng(seed);
  std::vector<uint8_t> in((size_t)K * rowlen);
  for (auto &b : in) b = (uint8_t)(rng() & 0xFF);
  const SharedLayout L = make_shared_layout(tab.cw, tab.psw, tab.slots, tab.table_bytes, 8);
  const uint32_t win = L.raw_bytes;  // 8-bit: one sample per byte
  const uint32_t cw = tab.cw, psw = tab.psw;
  auto sample = [&](uint32_t r, uint64_t ws, uint64_t pos) -> uint32_t {
    // bytes the bulk copy would not bring read as 0xFF (stale shared memory)
    if (pos - ws >= win || pos >= rowlen) return 0xFFu;
    return in[(size_t)r * rowlen + pos];
  };
  uint64_t checked = 0, stages = 0, partial_ops = 0;
  std::vector<uint32_t> copy((kStageRows * 4 + 1) * cw), part((2 * tab.slots + 3) * psw, 0);
  const size_t zrow = L.zero_copy;
  const size_t dummy0 = (size_t)L.dummy_word, dummy1 = dummy0 + 2 * psw;
  std::vector<uint8_t> written(part.size());
  for (uint32_t dt = 0; dt < tiles_d; dt++) {
    for (uint32_t tt = 0; tt < std::min(ntt, tiles_t); tt++) {
      const uint32_t t0 = tt * T;
      std::vector<uint32_t> acc((size_t)DB * T / 2, 0), tot((size_t)DB * T, 0);
      uint32_t since = 0;
      for (uint32_t s = tab.tile_stage[dt]; s < tab.tile_stage[dt + 1]; s++) {
        stages++;
        const SharedStage &st = tab.stages[s];
        if (st.pool % 8) return fail("pool alignment", s, st.pool, 0);
        if (st.table_bytes > tab.table_bytes || st.table_bytes % 16)
          return fail("table bytes", s, st.table_bytes, tab.table_bytes);
        const size_t tlen = st.table_bytes / 2;
        const uint16_t *tb = &tab.pool[st.pool];
        auto T16 = [&](size_t i) -> uint32_t {
          if (i >= tlen) throw i;
          return tb[i];
        };
        auto T32 = [&](size_t i) -> uint32_t { return T16(i) | (T16(i + 1) << 16); };
        try {
          const uint32_t nsub = T16(0), nrows = T16(1), nitems = T16(2);
          if (nsub != st.nsub || nrows != st.nrows || nitems != st.nitems || nsub < 1 ||
              nsub > (uint32_t)kSubMax || nrows > (uint32_t)kStageRows || nitems > kItemsMax)
            return fail("header", s, nsub, nrows);
          // expansion
          std::fill(copy.begin(), copy.end(), 0xA5A5A5A5u);
          std::fill(copy.begin() + zrow, copy.end(), 0u);
          uint32_t row_words[kStageRows] = {0};  // words the kernel expands per row
          for (uint32_t r = 0; r < nrows; r++) {
            const uint32_t q = (r >= T16(8 + 4 + 2)) + (r >= T16(8 + 8 + 2)) + (r >= T16(8 + 12 + 2));
            if (q != st.row_sub[r]) return fail("row subgroup", s, r, q);
            const uint32_t bm = T16(8 + 4 * q) | (T16(8 + 4 * q + 1) << 16);
            if (bm != st.bmin[q] || bm % 4) return fail("bmin", s, q, bm);
            const uint64_t ws = (t0 + bm) / 16 * 16;
            const uint32_t x0 = t0 + bm - (uint32_t)ws;
            if (x0 + 4 * cw + 8 > win) return fail("raw window", s, x0, win);
            const uint32_t cwk = std::min<uint32_t>(T16(3 + q), cw);
            if (cwk % 2) return fail("odd copy width", s, q, cwk);
            row_words[r] = cwk;
            for (uint32_t m = 0; m < 4; m++)
              for (uint32_t kk = 0; kk < cwk; kk++) {
                uint32_t w = 0;
                for (uint32_t i = 0; i < 4; i++)
                  w |= sample(st.row_first + r, ws, ws + x0 + 4 * kk + m + i) << (8 * i);
                copy[(r * 4 + m) * cw + kk] = w;
              }
          }
          // phase A
          std::fill(written.begin(), written.end(), 0);
          for (size_t w = 2 * tab.slots * psw; w < dummy0; w++) written[w] = 1;  // zero series
          auto rd = [&](uint32_t offb, uint32_t g, uint32_t &w) {
            if (offb % 4) return false;
            const uint32_t off = offb / 4;
            if (off == zrow) {  // the zero row
              if (g >= cw) return false;
              w = 0;
              return true;
            }
            if ((size_t)off + g >= copy.size()) return false;
            if ((off % cw) + g >= cw) return false;  // stays in its copy of its row
            if (off / (4 * cw) >= nrows) return false;
            if ((off % cw) + g >= row_words[off / (4 * cw)]) return false;  // expanded words only
            w = copy[off + g];
            return true;
          };
          for (uint32_t it = 0; it < nitems; it++) {
            const uint32_t item = T16(kTabItems + it), q = item >> 8, c = item & 0xFF;
            if (q >= nsub) return fail("item subgroup", s, it, q);
            const uint32_t pg = T16(8 + 4 * q + 3);
            if (pg % 8) return fail("program alignment", s, q, pg);
            const uint32_t n = T32(pg) & 0xFFFF, ng = T32(pg) >> 16;
            const uint32_t nA = T32(pg + 2) & 0xFFFF, nB = T32(pg + 2) >> 16;
            const uint32_t dA = T32(pg + 4), dB = T32(pg + 6);
            if (n < 1 || n > (uint32_t)kSharedRows) return fail("program rows", s, q, n);
            if (dB != 0xFFFFFFFFu && nA != nB) return fail("unequal halves", s, nA, nB);
            if (dB == 0xFFFFFFFFu && nA) return fail("micro-ops without chain B", s, q, nA);
            // both half-chains of every lane of the chunk
            for (uint32_t half = 0; half < 2; half++) {
              const uint32_t d0 = half ? dB : dA;
              if (half && d0 == 0xFFFFFFFFu) {
                if (nB) return fail("half B without start", s, q, nB);
                break;
              }
              uint32_t lo[32] = {0}, hi[32] = {0};
              for (uint32_t lane = 0; lane < 32; lane++) {
                const uint32_t g = std::min(c * 31 + lane, ng - 1);  // lanes past the series
                for (uint32_t e = 0; e < (uint32_t)kSharedRows; e++) {
                  uint32_t w;
                  const uint32_t ob = T32(pg + 8 + 16 * half + 2 * e);
                  if (e >= n && ob != 4 * zrow) return fail("row past n not the zero row", s, q, e);
                  if (!rd(ob, g, w)) return fail("copy read", s, q, e);
                  lo[lane] += prmt4140(w);
                  hi[lane] += prmt4342(w);
                }
                if (c * 31 + lane < ng) partial_ops += 4 * n;
              }
              auto store = [&](uint32_t dstb) {
                if (dstb % 4) return fail("dst alignment", s, q, dstb);
                const size_t dst = dstb / 4;
                const bool dummy = dst == dummy0;
                for (uint32_t lane = 0; lane < 31; lane++) {
                  const uint32_t g = c * 31 + lane;
                  if (g >= ng) continue;
                  const uint32_t nlo = lo[lane + 1];
                  const size_t c0 = dst + 2 * g, c1 = c0 + psw;
                  if (!dummy && (dst % (2 * psw) || c1 + 1 >= 2 * (size_t)tab.slots * psw))
                    return fail("series write", s, (long)dst, g);
                  if (2 * g + 1 >= psw || (dummy && c1 + 1 >= dummy1)) return fail("series length", s, (long)dst, g);
                  if (dummy) continue;
                  part[c0] = lo[lane];
                  part[c0 + 1] = hi[lane];
                  part[c1] = (lo[lane] >> 16) | (hi[lane] << 16);
                  part[c1 + 1] = (hi[lane] >> 16) | (nlo << 16);
                  written[c0] = written[c0 + 1] = written[c1] = 1;
                  written[c1 + 1] = g + 1 < ng ? 1 : 2;  // 2: neighbour past the series
                  for (uint32_t x : {lo[lane], hi[lane]})
                    if ((x & 0xFFFF) > 8 * 255 || (x >> 16) > 8 * 255)
                      return fail("lane range", s, g, x);
                }
                return 0;
              };
              if (store(d0)) return 1;
              const size_t u0 = pg + 40 + 8 * (half ? nA : 0);
              const uint32_t nu = half ? nB : nA;
              for (uint32_t i = 0; i < nu; i++) {
                const uint32_t o = T32(u0 + 8 * i), nw = T32(u0 + 8 * i + 2);
                const uint32_t dst = T32(u0 + 8 * i + 4);
                if (T32(u0 + 8 * i + 6) != (dst / 4 != dummy0 ? 1u : 0u))
                  return fail("store flag", s, q, i);
                for (uint32_t lane = 0; lane < 32; lane++) {
                  const uint32_t g = std::min(c * 31 + lane, ng - 1);
                  uint32_t wo, wn;
                  if (!rd(o, g, wo) || !rd(nw, g, wn)) return fail("chain read", s, q, i);
                  // lane-wise: the old sample is a summand, so no borrow
                  for (uint32_t sh = 0; sh < 32; sh += 16) {
                    if (((lo[lane] >> sh) & 0xFFFF) < ((prmt4140(wo) >> sh) & 0xFFFF) ||
                        ((hi[lane] >> sh) & 0xFFFF) < ((prmt4342(wo) >> sh) & 0xFFFF))
                      return fail("chain borrow", s, q, i);
                  }
                  lo[lane] = lo[lane] - prmt4140(wo) + prmt4140(wn);
                  hi[lane] = hi[lane] - prmt4342(wo) + prmt4342(wn);
                  if (c * 31 + lane < ng) partial_ops += 8;
                }
                if (store(dst)) return 1;
              }
            }
          }
          // phase B
          if (since + kSubMax > kLaneSeries) {
            for (size_t qq = 0; qq < acc.size(); qq++) {
              tot[2 * qq] += acc[qq] & 0xFFFF;
              tot[2 * qq + 1] += acc[qq] >> 16;
              acc[qq] = 0;
            }
            since = 0;
          }
          since += kSubMax;
          for (uint32_t j = 0; j < DB; j++)
            for (uint32_t q = 0; q < (uint32_t)kSubMax; q++) {
              const uint32_t offb = T32(kTabSeries + 2 * (j * kSubMax + q));
              if (offb % 4) return fail("series offset alignment", s, j, q);
              const uint32_t off = offb / 4;
              for (uint32_t i = 0; i < T / 2; i++) {
                const size_t w = (size_t)off + i;
                if (w >= dummy0) return fail("series read", s, j, i);
                if (written[w] != 1) return fail("unwritten series word", s, j, (long)w);
                const uint32_t a = acc[(size_t)j * (T / 2) + i] + part[w];
                if ((a & 0xFFFF) < (acc[(size_t)j * (T / 2) + i] & 0xFFFF) && (part[w] & 0xFFFF))
                  return fail("lane carry", s, j, i);
                acc[(size_t)j * (T / 2) + i] = a;
              }
            }
        } catch (size_t i) {
          return fail("table read past its end", s, (long)i, (long)tlen);
        }
      }
      for (size_t q = 0; q < acc.size(); q++) {
        tot[2 * q] += acc[q] & 0xFFFF;
        tot[2 * q + 1] += acc[q] >> 16;
      }
      // direct sums
      for (uint32_t j = 0; j < DB; j++) {
        const uint32_t d = dt * DB + j;
        if (d >= D) continue;
        for (uint32_t t = 0; t < T && t0 + t < S; t++) {
          uint32_t want = 0;
          for (uint32_t r = 0; r < K; r++)
            want += in[(size_t)r * rowlen + t0 + t + host_delay(first, step, d, shift[r])];
          if (tot[(size_t)j * T + t] != want) return fail("sum", d, t0 + t, (long)want);
          checked++;
        }
      }
    }
  }
  printf("PASS samples=%llu stages=%llu slots=%u cw=%u psw=%u smem=%zu table=%u adds_partial=%llu "
         "adds_series=%llu\n",
         (unsigned long long)checked, (unsigned long long)stages, tab.slots, cw, psw, tab.smem,
         tab.table_bytes, (unsigned long long)tab.adds_partial,
         (unsigned long long)tab.adds_series);
  return 0;
}

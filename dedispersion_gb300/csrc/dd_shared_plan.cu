// dd_shared_plan.cu -- host construction of the shared-partial-sum stage
// tables of a single-step plan.
//
// Per DM tile, the rows of a group are cut greedily into subgroups of up to
// kSharedRows consecutive rows, each as long as its distinct relative-delay
// vectors stay few enough to hold in shared memory and its relative delays
// stay below kRelMax.  Each subgroup's vectors are ordered into a chain
// (nearest neighbour in the number of rows that differ), and consecutive
// subgroups are packed into stages of at most kSubMax.  The delays are the
// reference's (include/Dedispersion.hpp:81): (uint)((firstDM + dm * dmStep)
// * shift), each operation rounded to float (this file is compiled with
// -ffp-contract=off), equal to dd::host_delay.
#include "dd_shared_plan.h"

#include <algorithm>
#include <array>
#include <cstdio>

#include "dd_shared.cuh"

namespace dd {

namespace {

constexpr uint32_t kRelMax = 124;  // relative delay within a subgroup (rel >> 2 <= 31)
constexpr uint32_t kNvCap = 32;    // vectors of one subgroup

uint32_t ceil_div(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

using Vec = std::array<uint8_t, kSharedRows>;

struct Sub {
  uint32_t r0 = 0, n = 0, bmin = 0, spread = 0, maxrel = 0;
  uint32_t hsum = 0;             // rows moved along the whole chain
  std::vector<Vec> vec;          // chain order
  std::vector<uint32_t> pos;     // per DM of the tile: chain position of its vector
  std::vector<uint32_t> boff;    // per DM: base - bmin
};

// Rows [r, r + n) over the tile's DMs: relative vectors and bases.
struct Window {
  uint32_t DB;
  std::vector<uint32_t> dl, base;  // dl[e * DB + j]
  std::vector<uint64_t> key, uniq;
  explicit Window(uint32_t db) : DB(db), dl(kSharedRows * db), base(db), key(db), uniq(db) {}
  // Distinct vector count of the first n rows (UINT32_MAX past kRelMax).
  uint32_t count(uint32_t n, uint32_t *maxrel) {
    for (uint32_t j = 0; j < DB; j++) {
      uint32_t b = UINT32_MAX;
      for (uint32_t e = 0; e < n; e++) b = std::min(b, dl[e * DB + j]);
      base[j] = b;
    }
    uint32_t mr = 0;
    for (uint32_t j = 0; j < DB; j++) {
      uint64_t kk = 0;
      for (uint32_t e = 0; e < n; e++) {
        const uint32_t rel = dl[e * DB + j] - base[j];
        mr = std::max(mr, rel);
        kk |= (uint64_t)(rel & 0xFFu) << (8 * e);
      }
      key[j] = kk;
    }
    *maxrel = mr;
    if (mr > kRelMax) return UINT32_MAX;
    // Neighbouring DMs mostly share a vector: drop runs first, then sort the
    // few keys left.
    uniq.clear();
    for (uint32_t j = 0; j < DB; j++)
      if (j == 0 || key[j] != key[j - 1]) uniq.push_back(key[j]);
    std::sort(uniq.begin(), uniq.end());
    uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
    return (uint32_t)uniq.size();
  }
};

uint32_t hamming(const Vec &a, const Vec &b, uint32_t n) {
  uint32_t h = 0;
  for (uint32_t e = 0; e < n; e++) h += a[e] != b[e];
  return h;
}

// Greedy subgroups of one DM tile with at most nv_cap vectors each.
std::vector<Sub> cut_tile(const std::vector<float> &row_shift, const float *dv, uint32_t DB,
                          uint32_t nv_cap) {
  const uint32_t K = (uint32_t)row_shift.size();
  std::vector<Sub> subs;
  Window w(DB);
  auto delay = [&](uint32_t r, uint32_t j) { return static_cast<uint32_t>(dv[j] * row_shift[r]); };
  uint32_t r = 0;
  while (r < K) {
    // The largest subgroup that fits: the vector count and the largest
    // relative delay only grow with the rows, so try all rows first and
    // search downwards only when they do not fit.
    const uint32_t mmax = std::min<uint32_t>(kSharedRows, K - r);
    for (uint32_t e = 0; e < mmax; e++)
      for (uint32_t j = 0; j < DB; j++) w.dl[e * DB + j] = delay(r + e, j);
    uint32_t mr = 0, counted = 0, nv = 0;  // the Window holds the count of `counted` rows
    auto fits = [&](uint32_t m) {
      nv = w.count(m, &mr);
      counted = m;
      return nv != UINT32_MAX && nv <= nv_cap;
    };
    uint32_t n = mmax;
    if (!fits(mmax)) {
      uint32_t lo = 1, hi = mmax;  // fits(lo) holds (one row, one vector), fits(hi) does not
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (fits(mid)) lo = mid; else hi = mid;
      }
      n = lo;
    }
    Sub s;
    s.r0 = r;
    s.n = n;
    if (counted != n) fits(n);
    s.maxrel = mr;
    uint32_t bmin = UINT32_MAX, bmax = 0;
    for (uint32_t j = 0; j < DB; j++) {
      bmin = std::min(bmin, w.base[j]);
      bmax = std::max(bmax, w.base[j]);
    }
    s.bmin = bmin & ~3u;
    s.spread = bmax - s.bmin;
    // vectors in first-appearance order, then the nearest-neighbour chain
    std::vector<uint32_t> first(nv, UINT32_MAX), vid(DB);
    std::vector<uint32_t> appear;  // vector id in appearance order
    for (uint32_t j = 0; j < DB; j++) {
      const uint32_t id =
          (uint32_t)(std::lower_bound(w.uniq.begin(), w.uniq.begin() + nv, w.key[j]) -
                     w.uniq.begin());
      vid[j] = id;
      if (first[id] == UINT32_MAX) {
        first[id] = (uint32_t)appear.size();
        appear.push_back(id);
      }
    }
    std::vector<Vec> by_id(nv);
    for (uint32_t id = 0; id < nv; id++)
      for (uint32_t e = 0; e < (uint32_t)kSharedRows; e++)
        by_id[id][e] = e < n ? (uint8_t)((w.uniq[id] >> (8 * e)) & 0xFFu) : 0;
    std::vector<uint32_t> chain_pos(nv, UINT32_MAX), left(appear.begin() + 1, appear.end());
    uint32_t cur = appear[0];
    chain_pos[cur] = 0;
    s.vec.push_back(by_id[cur]);
    while (!left.empty()) {
      size_t best = 0;
      uint32_t bh = UINT32_MAX;
      for (size_t i = 0; i < left.size(); i++) {
        const uint32_t h = hamming(by_id[cur], by_id[left[i]], n);
        if (h < bh) { bh = h; best = i; }
      }
      cur = left[best];
      s.hsum += bh;
      left.erase(left.begin() + best);
      chain_pos[cur] = (uint32_t)s.vec.size();
      s.vec.push_back(by_id[cur]);
    }
    s.pos.resize(DB);
    s.boff.resize(DB);
    for (uint32_t j = 0; j < DB; j++) {
      s.pos[j] = chain_pos[vid[j]];
      s.boff[j] = w.base[j] - s.bmin;
    }
    subs.push_back(std::move(s));
    r += n;
  }
  return subs;
}

std::string fmt(const char *f, unsigned long long a, unsigned long long b) {
  char buf[256];
  snprintf(buf, sizeof(buf), f, a, b);
  return buf;
}

}  // namespace

std::string build_shared_tables(const KernelInfo &k, const std::vector<float> &row_shift,
                                float first_dm, float dm_step, uint32_t nr_dms, uint32_t bits,
                                size_t smem_budget, SharedTables *out) {
  SharedTables &S = *out;
  S = SharedTables();
  const uint32_t T = k.tile_t, DB = k.tile_d, TY = (uint32_t)k.threads / 32;
  const uint32_t items_cap = std::min<uint32_t>(TY, kItemsMax);
  const uint32_t tiles_d = nr_dms ? ceil_div(nr_dms, DB) : 0;
  std::vector<float> dm_value((size_t)tiles_d * DB);
  for (size_t i = 0; i < dm_value.size(); i++) {
    const uint32_t dm = std::min((uint32_t)i, nr_dms ? nr_dms - 1 : 0);
    const float step_dm = static_cast<float>(dm) * dm_step;
    dm_value[i] = first_dm + step_dm;
  }
  uint32_t nv_cap = kNvCap;
  std::vector<std::vector<Sub>> tiles(tiles_d);
  for (;;) {
    uint32_t spread = 0, maxrel = 0, nv_max = 1;
    for (uint32_t t = 0; t < tiles_d; t++) {
      tiles[t] = cut_tile(row_shift, &dm_value[(size_t)t * DB], DB, nv_cap);
      for (const Sub &s : tiles[t]) {
        spread = std::max(spread, s.spread);
        maxrel = std::max(maxrel, s.maxrel);
        nv_max = std::max(nv_max, (uint32_t)s.vec.size());
      }
    }
    const uint32_t ng_max = ceil_div(spread + T + 2, 4) + 1;
    if (ceil_div(ng_max, 31) > kItemsMax)
      return fmt("DM spread of %llu samples per tile is too large (tile of %llu DMs); use "
                 "fewer DMs per tile", spread, DB);
    S.psw = std::max<uint32_t>(2 * ng_max, 64);  // the dummy series takes 32 lanes' junk stores
    S.cw = std::max<uint32_t>((maxrel / 4 + ng_max + 2 + 1) & ~1u, ng_max);  // zero row >= ng
    // Table size bound: header, items, series offsets, and kSubMax of the
    // largest program (80 bytes + 16 per micro-op, at most the chain's moved
    // rows).
    uint32_t prog_max = 0;
    for (uint32_t t = 0; t < tiles_d; t++)
      for (const Sub &s : tiles[t]) prog_max = std::max(prog_max, 80 + 16 * s.hsum);
    const uint32_t tbytes = 2 * kTabSeries + 16 * DB + kSubMax * (prog_max + 16);
    S.slots = 0;
    for (uint32_t sl = kSubMax * nv_cap; sl >= 1; sl--) {
      const SharedLayout L = make_shared_layout(S.cw, S.psw, sl, tbytes, bits);
      if (L.total <= smem_budget) {
        S.slots = sl;
        S.table_bytes = tbytes;
        S.smem = L.total;
        break;
      }
    }
    if (!S.slots)
      return fmt("partial sums of %llu samples do not fit %llu bytes of shared memory",
                 (unsigned long long)S.psw * 2, smem_budget);
    if (S.slots >= nv_max) break;
    nv_cap = S.slots;  // fewer rows per subgroup, so that one always fits
  }
  const SharedLayout L0 = make_shared_layout(S.cw, S.psw, S.slots, S.table_bytes, bits);
  const uint32_t zero_bytes = 4 * L0.zero_word, dummy_bytes = 4 * L0.dummy_word;
  const uint32_t zero_row = 4 * L0.zero_copy;  // copy-area byte offset of the zero row

  S.tile_stage.push_back(0);
  uint32_t tb_max = 16;
  for (uint32_t t = 0; t < tiles_d; t++) {
    const std::vector<Sub> &subs = tiles[t];
    size_t i = 0;
    while (i < subs.size()) {
      // Pack consecutive subgroups.
      size_t end = i + 1;
      uint32_t nv = (uint32_t)subs[i].vec.size(), rows = subs[i].n;
      uint32_t items = ceil_div(ceil_div(subs[i].spread + T + 2, 4) + 1, 31);
      while (end < subs.size() && end - i < (size_t)kSubMax) {
        const Sub &s = subs[end];
        const uint32_t it = ceil_div(ceil_div(s.spread + T + 2, 4) + 1, 31);
        if (nv + s.vec.size() > S.slots || items + it > items_cap || rows + s.n > kStageRows)
          break;
        nv += (uint32_t)s.vec.size();
        items += it;
        rows += s.n;
        end++;
      }
      const uint32_t nsub = (uint32_t)(end - i);
      while (S.pool.size() % 8) S.pool.push_back(0);
      const size_t at = S.pool.size();
      std::vector<uint16_t> tb(kTabSeries + 2 * kSubMax * DB, 0);
      auto put32 = [&](size_t u16_index, uint32_t v) {
        tb[u16_index] = (uint16_t)(v & 0xFFFFu);
        tb[u16_index + 1] = (uint16_t)(v >> 16);
      };
      auto push32 = [&](uint32_t v) {
        tb.push_back((uint16_t)(v & 0xFFFFu));
        tb.push_back((uint16_t)(v >> 16));
      };
      tb[0] = (uint16_t)nsub;
      tb[1] = (uint16_t)rows;
      SharedStage st{};
      st.pool = (uint32_t)at;
      st.row_first = subs[i].r0;
      st.nrows = (uint16_t)rows;
      st.nsub = (uint16_t)nsub;
      uint32_t rstart = 0, slot = 0, nitems = 0;
      for (uint32_t q = 0; q < (uint32_t)kSubMax; q++) {
        if (q >= nsub) {
          tb[8 + 4 * q + 2] = 0xFFFF;
          for (uint32_t j = 0; j < DB; j++) put32(kTabSeries + 2 * (j * kSubMax + q), zero_bytes);
          continue;
        }
        const Sub &s = subs[i + q];
        const uint32_t ng = ceil_div(s.spread + T + 2, 4) + 1;
        // copy words phase A reads in each of the subgroup's rows: rel >> 2 + g
        // for g < ng (even: the expansion writes word pairs)
        tb[3 + q] = (uint16_t)std::min<uint32_t>(((s.maxrel >> 2) + ng + 1) & ~1u, S.cw);
        tb[8 + 4 * q + 0] = (uint16_t)(s.bmin & 0xFFFFu);
        tb[8 + 4 * q + 1] = (uint16_t)(s.bmin >> 16);
        tb[8 + 4 * q + 2] = (uint16_t)rstart;
        st.bmin[q] = s.bmin;
        for (uint32_t e = 0; e < s.n; e++) st.row_sub[rstart + e] = (uint8_t)q;
        for (uint32_t c = 0; c < ceil_div(ng, 31); c++)
          tb[kTabItems + nitems++] = (uint16_t)(q << 8 | c);
        // series byte offsets of every DM: copy (base & 1), word (base >> 1)
        for (uint32_t j = 0; j < DB; j++) {
          const uint32_t b = s.boff[j];
          put32(kTabSeries + 2 * (j * kSubMax + q),
                4 * ((2 * (slot + s.pos[j]) + (b & 1u)) * S.psw + (b >> 1)));
        }
        // program
        while (tb.size() % 8) tb.push_back(0);
        tb[8 + 4 * q + 3] = (uint16_t)tb.size();
        auto off = [&](uint32_t e, uint32_t rel) {
          return 4 * ((rstart + e) * 4 * S.cw + (rel & 3u) * S.cw + (rel >> 2));
        };
        const uint32_t nvq = (uint32_t)s.vec.size();
        std::vector<uint32_t> h(nvq, 0);  // rows moved from vector v - 1 to v
        for (uint32_t v = 1; v < nvq; v++) h[v] = hamming(s.vec[v - 1], s.vec[v], s.n);
        // Half B starts at vector m (from scratch): balance the micro-ops.
        uint32_t m = nvq, best = UINT32_MAX;
        if (nvq >= 2) {
          uint32_t total = 0;
          for (uint32_t v = 1; v < nvq; v++) total += h[v];
          uint32_t pre = 0;  // micro-ops of A = sum h[1..m-1]
          for (uint32_t mm = 1; mm < nvq; mm++) {
            if (mm > 1) pre += h[mm - 1];
            const uint32_t b = total - pre - h[mm];
            const uint32_t cost = std::max(pre, b);
            if (cost < best) { best = cost; m = mm; }
          }
        }
        const bool hasB = m < nvq;
        auto dst_of = [&](uint32_t v) { return 4 * 2 * (slot + v) * S.psw; };
        std::vector<uint32_t> ua, ub;
        auto uops = [&](std::vector<uint32_t> &u, uint32_t from, uint32_t to) {
          for (uint32_t v = from + 1; v < to; v++) {
            uint32_t left = h[v];
            for (uint32_t e = 0; e < s.n; e++)
              if (s.vec[v - 1][e] != s.vec[v][e]) {
                u.push_back(off(e, s.vec[v - 1][e]));
                u.push_back(off(e, s.vec[v][e]));
                u.push_back(--left == 0 ? dst_of(v) : dummy_bytes);
                u.push_back(left == 0 ? 1u : 0u);  // 1: the store is real
              }
          }
        };
        uops(ua, 0, m);
        if (hasB) uops(ub, m, nvq);
        // Pad the shorter half with no-op micro-ops (zero row in and out,
        // result to the dummy series): the kernel steps both in lockstep.
        while (hasB && ua.size() < ub.size()) ua.insert(ua.end(), {zero_row, zero_row, dummy_bytes, 0});
        while (hasB && ub.size() < ua.size()) ub.insert(ub.end(), {zero_row, zero_row, dummy_bytes, 0});
        push32(s.n | ng << 16);
        push32((uint32_t)(ua.size() / 4) | (uint32_t)(ub.size() / 4) << 16);
        push32(dst_of(0));
        push32(hasB ? dst_of(m) : 0xFFFFFFFFu);
        for (uint32_t e = 0; e < (uint32_t)kSharedRows; e++)
          push32(e < s.n ? off(e, s.vec[0][e]) : zero_row);
        for (uint32_t e = 0; e < (uint32_t)kSharedRows; e++)
          push32(hasB && e < s.n ? off(e, s.vec[m][e]) : zero_row);
        for (uint32_t w : ua) push32(w);
        for (uint32_t w : ub) push32(w);
        const uint64_t row_ops = kSharedRows * (hasB ? 2u : 1u) + 2 * (ua.size() + ub.size()) / 4;
        S.adds_partial += row_ops * 4 * ng;
        S.adds_series += (uint64_t)DB * T;
        slot += nvq;
        rstart += s.n;
      }
      tb[2] = (uint16_t)nitems;
      while (tb.size() % 8) tb.push_back(0);
      st.nitems = (uint16_t)nitems;
      if (tb.size() * 2 > 65535) return fmt("stage table of %llu bytes (limit %llu)", tb.size() * 2, 65535);
      st.table_bytes = (uint16_t)(tb.size() * 2);
      tb_max = std::max<uint32_t>(tb_max, st.table_bytes);
      S.pool.insert(S.pool.end(), tb.begin(), tb.end());
      S.stages.push_back(st);
      i = end;
    }
    S.tile_stage.push_back((uint32_t)S.stages.size());
  }
  if (tb_max > S.table_bytes)
    return fmt("stage table of %llu bytes exceeds its bound of %llu", tb_max, S.table_bytes);
  // Table slots sized to the largest actual table; every stage copies that
  // many bytes, so the pool ends with one table's worth of zeros.
  S.table_bytes = tb_max;
  S.pool.insert(S.pool.end(), tb_max / 2, 0);
  S.smem = make_shared_layout(S.cw, S.psw, S.slots, tb_max, bits).total;
  return "";
}

}  // namespace dd

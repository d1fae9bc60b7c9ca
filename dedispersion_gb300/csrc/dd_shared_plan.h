// dd_shared_plan.h -- host construction of the shared-partial-sum stage
// tables (dd_shared.cuh describes the kernel that reads them).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "dd_internal.h"

namespace dd {

struct SharedTables {
  std::vector<SharedStage> stages;   // all DM tiles, tile by tile
  std::vector<uint32_t> tile_stage;  // [tiles_d + 1]
  std::vector<uint16_t> pool;        // stage tables
  uint32_t cw = 0, psw = 0, slots = 0, table_bytes = 0;
  size_t smem = 0;
  // Integer adds of one (group, time tile) over all DM tiles: partial sums
  // (first vectors' rows and the chains' moved rows, each add or subtract
  // counted) and series adds.
  uint64_t adds_partial = 0, adds_series = 0;
};

// Builds the tables of a single-step problem for kernel `k` (family
// kFamilyShared8).  `row_shift` holds each row's delay per unit DM in the
// order of a group's entries.  Returns "" on success, else why the shape
// does not fit this kernel (shared memory, 16-bit offsets).
std::string build_shared_tables(const KernelInfo &k, const std::vector<float> &row_shift,
                                float first_dm, float dm_step, uint32_t nr_dms, uint32_t bits,
                                size_t smem_budget, SharedTables *out);

}  // namespace dd

// Host-side graph container shared by the generator, the COO readers and the
// C ABI.  Blocks are CSR with int64 row offsets and int32 columns.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "mmsb.h"

struct HostCsr {
  int64_t n_rows = 0, n_cols = 0;
  std::vector<int64_t> row_ptr;  // n_rows + 1
  std::vector<int32_t> col;      // nnz
  std::vector<float> val;        // empty: binary
  int64_t nnz() const { return (int64_t)col.size(); }
  mmsb_csr view() const;
};

struct mmsb_host_graph {
  int64_t part[4] = {0, 0, 0, 0};  // n_X, n_A, n_B, n_C
  int64_t n_edges = 0;
  int n_blocks = 0;
  HostCsr blocks[MMSB_NUM_BLOCKS];
  int32_t k = 0;
  std::vector<float> pi;  // k x N column-major ground truth (optional)
};

// Builds CSR from (row, col, val) triplets; duplicates summed (sum_dups) or
// collapsed to one entry; columns sorted within each row.
HostCsr csr_from_triplets(int64_t n_rows, int64_t n_cols, std::vector<int64_t>& rows,
                          std::vector<int32_t>& cols, std::vector<float>* vals,
                          bool sum_dups);

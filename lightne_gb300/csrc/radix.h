// Device sorts of the sparsifier: the radix sort and partitions of its
// samples, and the row sort of the hash-range rounds' CSR.
#pragma once
#include <stdint.h>

#include "lne_internal.h"

namespace lne {

// Sorts `count` (key, value) pairs by the low `key_bits` bits of the key,
// stably, in ceil(key_bits / 8) passes on ctx->stream, and writes the result
// as CSR columns (key & col_mask, int32) and values (value bits as float).
// keys/vals are overwritten; keys_tmp/vals_tmp are scratch of the same size.
// Bits of the key above key_bits must be zero.  Launches are added to
// *launches when it is not NULL.
int radix_sort_pairs_to_csr(lne_ctx* ctx, unsigned long long* keys, uint32_t* vals, unsigned long long* keys_tmp,
                            uint32_t* vals_tmp, int64_t count, int key_bits, unsigned long long col_mask,
                            int32_t* out_col, float* out_val, int* launches);

// The symmetric CSR from `count` upper-triangle items (u << cbits | v with
// u <= v, float bits): a stable LSD sort by (u, v) whose last pass writes
// each entry (u, v) to out_col/out_val at upoff[u] + its sorted position and
// its transpose (v << cbits | u) to the scratch buffers, then a stable sort
// of the transposes by v (ceil(cbits / 8) passes) whose last pass writes
// each off-diagonal (v, u) at looff[v] + its sorted position.  upoff/looff
// place a row's lower entries before its diagonal and upper ones; nnz
// bounds the positions (kFlagSortOverflow otherwise).  keys/vals are
// overwritten; keys_tmp/vals_tmp are scratch of the same size.
int radix_sort_sym_csr(lne_ctx* ctx, unsigned long long* keys, uint32_t* vals, unsigned long long* keys_tmp,
                       uint32_t* vals_tmp, int64_t count, int cbits, const int64_t* upoff, const int64_t* looff,
                       int64_t nnz, int32_t* out_col, float* out_val, int* launches);

// Reorders `count` pair keys by the top min(8, table_bits) bits of their
// pair-table slot (hash64_2(key) & (2^table_bits - 1)) into `out`, so that
// consecutive inserts touch one slice of the table.  Stable.
int partition_by_slot(lne_ctx* ctx, const unsigned long long* keys, unsigned long long* out, int64_t count,
                      int table_bits, int* launches);

// Stable LSD sort of `count` words by their top `top_bits` bits (0..24; 0
// is a no-op), ping-ponging between keys and tmp; *result is set to the
// buffer that holds the sorted words.
int partition_by_top_bits(lne_ctx* ctx, unsigned long long* keys, unsigned long long* tmp, int64_t count,
                          int top_bits, unsigned long long** result, int* launches);

// Sorts every row of a CSR by column: row r's entries are
// (scol, sval)[row_ptr[r] .. row_ptr[r + 1]) in any order, with distinct
// columns in [0, ncols); they are written in column order at the same
// positions of (dcol, dval).  scol == dcol and sval == dval sort in place.
// Rows of at most ctx->row_sort_warp_max entries are sorted by one warp in
// registers, longer ones by a thread block through a shared-memory bitmap of
// the column range.  A repeated or out-of-range column sets
// kFlagSortOverflow.  Defined in csr_rows.cu.
int sort_csr_rows(lne_ctx* ctx, const int64_t* row_ptr, int64_t n, int64_t ncols, const int32_t* scol,
                  const float* sval, int32_t* dcol, float* dval, int* launches);

}  // namespace lne

// qeg_sort.h -- stable LSD radix sort of (hi, lo, val) items by (hi, lo).
//
// Used by the as-of join to order its build side by (partition slot,
// timestamp) the way the reference's Sort does (a stable sort: equal keys keep
// their input order, ops/sort.cpp:93-100).
#pragma once

#include "qeg_internal.h"

namespace qeg {

struct SortItems {
  uint64_t* lo;   // least significant key word
  uint32_t* hi;   // most significant key word
  uint32_t* val;  // payload
};

// Sorts n items ascending by (hi, lo) over the low `lo_bits` bits of lo and the
// low `hi_bits` bits of hi (higher bits must be zero), stably: items with
// equal keys keep their order. `a` holds the input, `b` is scratch of the same
// size; returns whichever of the two holds the result. 8-bit digits, one
// histogram + scan + scatter per digit.
SortItems radix_sort_items(qeg_ctx* ctx, SortItems a, SortItems b, uint64_t n, int lo_bits, int hi_bits);

}  // namespace qeg

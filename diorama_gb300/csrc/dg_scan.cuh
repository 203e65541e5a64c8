// Internal entry points of the scan and the sort, shared by the tile stage and
// densification.
#pragma once
#include "dg_common.cuh"

namespace dg {

// Exclusive scan of min(*count, capacity) values of data in place (count may be
// NULL: all capacity values); total[0] gets the sum. scratch holds
// scan_scratch_bytes(capacity) bytes and is cleared by each launch. With gather,
// value j is source[gather[j]] instead and data only receives the scan.
size_t scan_scratch_bytes(uint32_t capacity);
dg_status scan_launch(dg_context* ctx, uint32_t* data, uint32_t capacity, const uint32_t* count, uint32_t* total,
                      void* scratch, const uint32_t* gather = nullptr, const uint32_t* source = nullptr);

// Stable LSD radix sort with the reference's pass plan, in place in keys/values
// (the scratch pair holds the odd passes). key_words = 1 for u32 keys, 2 for u64
// keys stored (low, high) whose high word contributes high_bits bits.
struct SortPlan {
  uint32_t capacity;
  uint32_t key_words;
  uint32_t high_bits;
  uint32_t passes;     // even in the reference's plans, so the result lands back in keys/values
  uint32_t shift[8];   // bit offset of each pass's 8-bit digit within the key
  bool narrow_last;    // the key's bits above the last pass's low 4 are all zero: a 4-bit last pass
};
SortPlan sort_plan(uint32_t capacity, uint32_t high_bits);
// u32 keys of which only the low `bits` bits vary (bits a multiple of 16).
SortPlan sort_plan_low_bits(uint32_t capacity, uint32_t bits);
// The fewest 8-bit passes for keys whose varying bits are the low `bits` (u32
// keys) or all 32 low-word bits plus `bits` high-word bits (u64 keys). With an
// odd number of passes the result lands in keys_alt/values_alt.
SortPlan sort_plan_digits(uint32_t capacity, uint32_t key_words, uint32_t bits);
// Tells a plan that only the key's low `bits` bits (of the low and high words
// together) vary; its last pass then sorts a 4-bit digit when that covers them.
void sort_plan_key_bits(SortPlan& p, uint32_t bits);
// Per-device kernel attributes; called once when a context is created.
dg_status sort_init();
size_t sort_scratch_bytes(const SortPlan& plan);
dg_status sort_launch(dg_context* ctx, const SortPlan& plan, void* keys, uint32_t* values, void* keys_alt,
                      uint32_t* values_alt, const uint32_t* count, void* scratch);

}  // namespace dg

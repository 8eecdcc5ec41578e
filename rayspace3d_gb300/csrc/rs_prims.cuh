// rs_prims.cuh -- host entry points of the engine's device primitives.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "rs_launch.cuh"

namespace rs {

// Stable LSD radix sort of 64-bit keys (and optional 32-bit values) on bits
// [begin_bit, end_bit), 8 bits per pass, in place; n < 2^32.  Temporaries come from the
// library's memory pool.  A pass whose bounded look-back wait ran out ORs err_bit into
// *err (a device word; null = the library's word, read with sort_error_read): the
// result is then invalid.
cudaError_t radix_sort_u64(uint64_t* keys, uint32_t* vals, size_t n, int end_bit, cudaStream_t s,
                           int begin_bit = 0, uint32_t* err = nullptr, uint32_t err_bit = 1);
// The same sort over caller scratch of radix_sort_scratch_bytes (256-byte aligned): no
// pool allocation, one memset.  With hist_ready the caller has already written, into
// radix_sort_hist(scratch, ...), the counts of every digit of every pass (hist[p * 256 + d],
// 8-bit digits from begin_bit), and the sort does not read the keys for them.
size_t radix_sort_scratch_bytes(size_t n, int end_bit, int begin_bit, bool vals);
uint32_t* radix_sort_hist(void* scratch, size_t n, bool vals);
cudaError_t radix_sort_u64_in(uint64_t* keys, uint32_t* vals, size_t n, int end_bit, cudaStream_t s, int begin_bit,
                              uint32_t* err, uint32_t err_bit, void* scratch, bool hist_ready);
// Queues a copy of the library's sort error word (nonzero after a failed sort) to h_word.
cudaError_t sort_error_read(uint32_t* h_word, cudaStream_t s);
cudaError_t sort_error_clear(cudaStream_t s);

// Full 64-bit ascending sort of keys: a single-block bitonic sort for small inputs,
// the radix sort otherwise.
cudaError_t sort_u64_any(uint64_t* keys, size_t n, cudaStream_t s);
// Largest n of table_keys_sorted_small.
constexpr uint64_t kSmallTableSort = 4096;
// The n keys of a hash table (slots not equal to `empty`) into out[0..n), ascending by the
// key with its halves swapped when swap (and written that way back), else by the key:
// a gather kernel and a one-block sort, no host wait.  n <= kSmallTableSort; counter is
// one device word of scratch.
cudaError_t table_keys_sorted_small(const uint64_t* slots, uint64_t capacity, uint64_t empty, int swap, uint64_t* out,
                                    uint64_t n, unsigned long long* counter, cudaStream_t s);

// Exclusive prefix sums.  `total` (device, nullable) receives the sum of all inputs.
cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n, uint32_t* total, cudaStream_t s);
cudaError_t exclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, size_t n, int64_t* total, cudaStream_t s);

// Ordered stream compaction of a u64 array: copies every element != skip, in
// index order, to out; *count (device) receives how many were written.
cudaError_t compact_u64(const uint64_t* in, size_t n, uint64_t skip, uint64_t* out, uint64_t* count,
                        cudaStream_t s);

// Remove consecutive duplicates of a sorted u64 array in place; *count (device)
// receives the new length.
cudaError_t unique_sorted_u64(uint64_t* keys, size_t n, uint64_t* count, cudaStream_t s);

// Number of thread blocks of a launch that keeps every SM busy.
int sm_count();

}  // namespace rs

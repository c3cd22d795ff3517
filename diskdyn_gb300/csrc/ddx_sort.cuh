// Device-wide radix sort and scan (ddx_sort.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ddx {

// 32-bit words of temporary storage radix_sort_pairs / exclusive_scan need for n items.
size_t sort_temp_words(int n);
size_t scan_temp_words(int n);

// Stable ascending sort of (keys, vals) in place by the low key_bits bits of the keys.
cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, int n, int key_bits, uint32_t* temp,
                             cudaStream_t st);

// out[i] = sum of in[0..i-1]; *total (device, optional) = sum of all.  in == out allowed.
cudaError_t exclusive_scan(const uint32_t* in, uint32_t* out, int n, uint32_t* temp, uint32_t* total,
                           cudaStream_t st);

}  // namespace ddx

// Device-wide exclusive scan (ddx_scan.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ddx {

// 32-bit words of temporary storage exclusive_scan needs for n items.
size_t scan_temp_words(int n);

// out[i] = sum of in[0..i-1]; *total (device, optional) = sum of all.  in == out allowed.
cudaError_t exclusive_scan(const uint32_t* in, uint32_t* out, int n, uint32_t* temp, uint32_t* total,
                           cudaStream_t st);

// The same over strided arrays: element k is in[k * is] and out[k * os]; with copy, also
// copy[k * os] = in[k * is] (out and copy may be two fields of an array of structs, which then
// holds {start, size} pairs).
cudaError_t exclusive_scan_strided(const uint32_t* in, int is, uint32_t* out, int os, int n, uint32_t* temp,
                                   uint32_t* total, cudaStream_t st, uint32_t* copy);

}  // namespace ddx

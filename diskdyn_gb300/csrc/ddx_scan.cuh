// Device-wide exclusive scan (ddx_scan.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ddx {

// 32-bit words of temporary storage the scans need for n items.
size_t scan_temp_words(int n);

// out[i] = sum of in[0..i-1]; *total (device, optional) = sum of all.  in and out must not
// overlap.
cudaError_t exclusive_scan(const uint32_t* in, uint32_t* out, int n, uint32_t* temp, uint32_t* total,
                           cudaStream_t st);

// The same, written as 16-byte entries table[i] = {start, size = in[i], 0, 0} (a bucket
// table: the last two words are free for the caller).
cudaError_t exclusive_scan_table(const uint32_t* in, uint4* table, int n, uint32_t* temp, uint32_t* total,
                                 cudaStream_t st);

}  // namespace ddx

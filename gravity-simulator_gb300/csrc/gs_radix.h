// gs_radix.h -- stable LSD radix sort of (uint64 key, int32 value) pairs on
// the device (k_radix.cu).
#pragma once

#include "gs_internal.h"

namespace gs {

class RadixSorter {
  public:
    // Scratch for up to `cap` elements.
    ErrorStatus reserve(int cap);
    // Sorts keys/vals in place by the low key_bits bits (stable).  The
    // element count is read from device memory (*d_n <= max_n <= reserved
    // capacity; max_n sizes the launches).  A look-back wait that ran out
    // sets ST_WAIT_TIMEOUT in *status.
    ErrorStatus sort(uint64_t *keys, int *vals, const int *d_n, int max_n, int key_bits,
                     unsigned *status, cudaStream_t s);
    // 8-bit passes, an even number of them (the result lands back in keys).
    static int passes_for(int key_bits)
    {
        const int p = (key_bits + 7) / 8;
        return p + (p & 1);
    }
    // kernels per sort: histograms, digit bases, one per pass
    static int launches(int key_bits) { return 2 + passes_for(key_bits); }

  private:
    int capacity_ = 0, tiles_ = 0, sm_count_ = 1;
    DBuf hist_, lookback_, tmp_keys_, tmp_vals_;
};

}  // namespace gs

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
    // element count is read from device memory (*d_n <= reserved capacity).
    ErrorStatus sort(uint64_t *keys, int *vals, const int *d_n, int key_bits, cudaStream_t s);
    static int launches(int key_bits)
    {
        int p = (key_bits + 7) / 8;
        return 3 * (p + (p & 1));
    }

  private:
    int capacity_ = 0, tiles_ = 0;
    DBuf counts_, totals_, tmp_keys_, tmp_vals_;
};

}  // namespace gs

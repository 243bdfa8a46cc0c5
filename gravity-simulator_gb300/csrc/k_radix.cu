// k_radix.cu -- stable LSD radix sort of (uint64 key, int32 value) pairs.
//
// Replaces radix_sort_particles_morton_index (src/linear_octree.c:216-326).
// Any stable sort by the full key gives the same order as the reference's
// 9-bit LSD passes, so this sort uses 8-bit digits, one kernel per pass
// (a one-sweep radix sort with decoupled look-back, after Adinets and
// Merrill, "Onesweep: A Faster Least Significant Digit Radix Sort for GPUs",
// 2022; the look-back is Merrill and Garland's single-pass prefix scan,
// 2016):
//   1. k_radix_hist   -- one read of the keys: the digit histograms of every
//                        pass (a digit's count does not depend on the order);
//   2. k_radix_bases  -- per pass, the exclusive scan over digits: where each
//                        digit's run starts in the output;
//   3. k_radix_onesweep, once per pass -- a CTA takes the next tile of 4096
//      elements (tile order = start order, from an atomic counter), ranks
//      them stably by warp match (each warp owns 512 consecutive elements,
//      16 rounds of 32, ranked in index order), publishes its per-digit
//      counts, then for each digit walks back over the preceding tiles'
//      published counts / inclusive prefixes until it meets a prefix, and
//      writes the tile out through shared memory in digit order (coalesced
//      runs).  A pass reads and writes 12 bytes per element once.
// A tile waits only on tiles that started before it, so the waits end; each
// wait is still bounded in time (kWaitLimitNs): on expiry the CTA sets
// ST_WAIT_TIMEOUT in the caller's status word, publishes what it has and
// goes on, and the caller reports the failed sort.
// The element count is read from device memory, so a sort sits inside a
// CUDA graph even when the count is produced on the device (tree nodes).
#include "gs_internal.h"
#include "gs_ptx.cuh"
#include "gs_radix.h"

#include <algorithm>
#include <utility>

namespace gs {

constexpr int RX_THREADS = 256;
constexpr int RX_ITEMS = 16;
constexpr int RX_TILE = RX_THREADS * RX_ITEMS;   // 4096
constexpr int RX_WARPS = RX_THREADS / 32;
constexpr int RX_MAX_PASSES = 8;
constexpr int RX_LOOKBACK = 8;   // predecessor tiles read per look-back round

// Look-back words: two flag bits over a 62-bit count.
constexpr unsigned long long LB_AGGREGATE = 1ull << 62;   // the tile's own count
constexpr unsigned long long LB_PREFIX = 2ull << 62;      // count of this and all earlier tiles
constexpr unsigned long long LB_COUNT = (1ull << 62) - 1ull;

__global__ void __launch_bounds__(RX_THREADS)
k_radix_hist(const uint64_t *__restrict__ keys, const int *__restrict__ d_n, int passes,
             unsigned *__restrict__ hist)
{
    __shared__ unsigned h[RX_MAX_PASSES][256];
    for (int i = threadIdx.x; i < RX_MAX_PASSES * 256; i += RX_THREADS) (&h[0][0])[i] = 0u;
    __syncthreads();
    const int n = *d_n;
    for (int e = blockIdx.x * RX_THREADS + threadIdx.x; e < n; e += gridDim.x * RX_THREADS) {
        const uint64_t k = keys[e];
        for (int p = 0; p < passes; ++p) atomicAdd(&h[p][(unsigned)(k >> (8 * p)) & 255u], 1u);
    }
    __syncthreads();
    for (int p = 0; p < passes; ++p) {
        const unsigned c = h[p][threadIdx.x];
        if (c) atomicAdd(&hist[p * 256 + threadIdx.x], c);
    }
}

// hist[p][d] <- number of elements of pass p with a digit below d.
__global__ void __launch_bounds__(256) k_radix_bases(unsigned *__restrict__ hist, int passes)
{
    __shared__ unsigned wsum[8];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    for (int p = 0; p < passes; ++p) {
        const unsigned c = hist[p * 256 + t];
        unsigned incl = c;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        unsigned before = 0;
        for (int w = 0; w < warp; ++w) before += wsum[w];
        hist[p * 256 + t] = before + incl - c;
        __syncthreads();
    }
}

__device__ __forceinline__ unsigned long long ld_volatile(const unsigned long long *p)
{
    return *reinterpret_cast<const volatile unsigned long long *>(p);
}

__device__ __forceinline__ void st_volatile(unsigned long long *p, unsigned long long v)
{
    *reinterpret_cast<volatile unsigned long long *>(p) = v;
}

__global__ void __launch_bounds__(RX_THREADS)
k_radix_onesweep(const uint64_t *__restrict__ keys_in, const int *__restrict__ vals_in,
                 uint64_t *__restrict__ keys_out, int *__restrict__ vals_out,
                 const int *__restrict__ d_n, int shift, const unsigned *__restrict__ base,
                 unsigned long long *__restrict__ lookback, int *__restrict__ tile_ctr,
                 unsigned *__restrict__ status)
{
    __shared__ unsigned whist[RX_WARPS][256];
    __shared__ unsigned tile_off[256];     // output position of the tile's first element of digit d
    __shared__ unsigned local_start[256];  // position of digit d's run within the tile
    __shared__ unsigned wsum[RX_WARPS];
    __shared__ uint64_t stage[RX_TILE];    // the tile in digit order (keys, then values)
    __shared__ int s_tile;
    if (threadIdx.x == 0) s_tile = atomicAdd(tile_ctr, 1);
    for (int d = threadIdx.x; d < RX_WARPS * 256; d += RX_THREADS) (&whist[0][0])[d] = 0u;
    __syncthreads();
    const int tile = s_tile;
    const int n = *d_n;
    if (tile * RX_TILE >= n) return;   // block-uniform: no later tile waits on it
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;

    const int wbase = tile * RX_TILE + warp * (RX_ITEMS * 32);
    uint64_t key[RX_ITEMS];
    int val[RX_ITEMS];
    unsigned rank[RX_ITEMS];
    unsigned dig[RX_ITEMS];
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < RX_ITEMS; ++r) {
        const int e = wbase + r * 32 + lane;
        const bool in = e < n;
        key[r] = in ? keys_in[e] : 0ull;
        val[r] = in ? vals_in[e] : 0;
        dig[r] = in ? ((unsigned)(key[r] >> shift) & 255u) : 256u + lane;   // unique if out
        const unsigned peers = __match_any_sync(0xffffffffu, dig[r]);
        const int leader = __ffs(peers) - 1;
        unsigned before = 0;
        if (lane == leader && in) {
            before = whist[warp][dig[r]];
            whist[warp][dig[r]] = before + __popc(peers);
        }
        before = __shfl_sync(0xffffffffu, before, leader);
        rank[r] = before + __popc(peers & lt);
        __syncwarp();
    }
    __syncthreads();
    // thread d owns digit d: exclusive prefix over the warps, the tile's count
    const int d = threadIdx.x;
    unsigned count = 0;
    for (int w = 0; w < RX_WARPS; ++w) {
        const unsigned c = whist[w][d];
        whist[w][d] = count;
        count += c;
    }
    unsigned long long *mine = lookback + (size_t)tile * 256 + d;
    unsigned long long excl = 0;
    if (tile == 0) {
        st_volatile(mine, LB_PREFIX | count);
    } else {
        st_volatile(mine, LB_AGGREGATE | count);
        // Walk back over the preceding tiles, RX_LOOKBACK of them per round
        // (independent loads in flight together): add aggregates until a
        // prefix; a tile that has published nothing yet is re-read from
        // there.  Tile 0 always publishes a prefix, so j never passes it.
        int j = tile - 1;
        const unsigned long long t0 = global_ns();
        for (;;) {
            unsigned long long v[RX_LOOKBACK];
#pragma unroll
            for (int q = 0; q < RX_LOOKBACK; ++q)
                v[q] = j - q >= 0 ? ld_volatile(lookback + (size_t)(j - q) * 256 + d) : LB_PREFIX;
            int q = 0;
            bool done = false;
#pragma unroll
            for (int u = 0; u < RX_LOOKBACK; ++u) {
                if (q != u) continue;   // an earlier slot stopped the scan
                if (v[u] & LB_PREFIX) {
                    excl += v[u] & LB_COUNT;
                    done = true;
                } else if (v[u] & LB_AGGREGATE) {
                    excl += v[u] & LB_COUNT;
                    ++q;
                }
            }
            if (done) break;
            j -= q;
            if (q == 0) {
                if (global_ns() - t0 > kWaitLimitNs) {
                    atomicOr(status, ST_WAIT_TIMEOUT);
                    break;
                }
                __nanosleep(32);
            }
        }
        st_volatile(mine, LB_PREFIX | ((excl + count) & LB_COUNT));
    }
    tile_off[d] = base[d] + (unsigned)excl;
    // exclusive scan of the tile's digit counts: where each digit's run
    // starts when the tile is laid out in digit order
    {
        unsigned incl = count;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        unsigned before = 0;
        for (int w = 0; w < warp; ++w) before += wsum[w];
        local_start[d] = before + incl - count;
    }
    __syncthreads();
    // The tile goes through shared memory in digit order, so that
    // consecutive threads write consecutive output slots of a digit's run
    // (coalesced) instead of scattering element by element.
    const int valid = min(RX_TILE, n - tile * RX_TILE);
    unsigned lpos[RX_ITEMS];
#pragma unroll
    for (int r = 0; r < RX_ITEMS; ++r) {
        const int e = wbase + r * 32 + lane;
        lpos[r] = 0;
        if (e < n) {
            const unsigned dg = dig[r];
            lpos[r] = local_start[dg] + whist[warp][dg] + rank[r];
            stage[lpos[r]] = key[r];
        }
    }
    __syncthreads();
    unsigned dst[RX_ITEMS];
#pragma unroll
    for (int r = 0; r < RX_ITEMS; ++r) {
        const int i = r * RX_THREADS + threadIdx.x;
        dst[r] = 0;
        if (i < valid) {
            const uint64_t k = stage[i];
            const unsigned dg = (unsigned)(k >> shift) & 255u;
            dst[r] = tile_off[dg] + (unsigned)i - local_start[dg];
            keys_out[dst[r]] = k;
        }
    }
    __syncthreads();
    int *vstage = reinterpret_cast<int *>(stage);
#pragma unroll
    for (int r = 0; r < RX_ITEMS; ++r) {
        const int e = wbase + r * 32 + lane;
        if (e < n) vstage[lpos[r]] = val[r];
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RX_ITEMS; ++r) {
        const int i = r * RX_THREADS + threadIdx.x;
        if (i < valid) vals_out[dst[r]] = vstage[i];
    }
}

ErrorStatus RadixSorter::reserve(int cap)
{
    if (cap <= capacity_) return ok();
    const DeviceInfo *dev = nullptr;
    GS_TRY(device_info(&dev));
    sm_count_ = dev->sm_count;
    capacity_ = cap;
    tiles_ = (cap + RX_TILE - 1) / RX_TILE;
    GS_TRY(hist_.reserve((size_t)(RX_MAX_PASSES * 256 + RX_MAX_PASSES) * sizeof(unsigned)));
    GS_TRY(lookback_.reserve((size_t)RX_MAX_PASSES * tiles_ * 256 * sizeof(unsigned long long)));
    GS_TRY(tmp_keys_.reserve((size_t)cap * sizeof(uint64_t)));
    GS_TRY(tmp_vals_.reserve((size_t)cap * sizeof(int)));
    return ok();
}

ErrorStatus RadixSorter::sort(uint64_t *keys, int *vals, const int *d_n, int max_n, int key_bits,
                              unsigned *status, cudaStream_t s)
{
    if (max_n > capacity_)
        return GS_RAISE(GRAV_VALUE_ERROR, "radix sort: %d elements exceed the capacity %d", max_n,
                        capacity_);
    const int passes = passes_for(key_bits);
    if (passes > RX_MAX_PASSES) return GS_RAISE(GRAV_VALUE_ERROR, "radix sort keys wider than 64 bits");
    if (max_n <= 0) return ok();
    const int tiles = (max_n + RX_TILE - 1) / RX_TILE;
    unsigned *hist = hist_.as<unsigned>();
    int *tile_ctr = reinterpret_cast<int *>(hist + RX_MAX_PASSES * 256);
    GS_CUDA(cudaMemsetAsync(hist_.p, 0, (size_t)(RX_MAX_PASSES * 256 + RX_MAX_PASSES) * sizeof(unsigned),
                            s));
    GS_CUDA(cudaMemsetAsync(lookback_.p, 0,
                            (size_t)passes * tiles * 256 * sizeof(unsigned long long), s));
    k_radix_hist<<<std::min(tiles, sm_count_ * 4), RX_THREADS, 0, s>>>(keys, d_n, passes, hist);
    k_radix_bases<<<1, 256, 0, s>>>(hist, passes);
    uint64_t *kin = keys, *kout = tmp_keys_.as<uint64_t>();
    int *vin = vals, *vout = tmp_vals_.as<int>();
    for (int p = 0; p < passes; ++p) {
        k_radix_onesweep<<<tiles, RX_THREADS, 0, s>>>(
            kin, vin, kout, vout, d_n, 8 * p, hist + 256 * p,
            lookback_.as<unsigned long long>() + (size_t)p * tiles * 256, tile_ctr + p, status);
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    GS_CUDA(cudaGetLastError());
    return ok();
}

}  // namespace gs

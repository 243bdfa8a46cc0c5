// k_radix.cu -- stable LSD radix sort of (uint64 key, int32 value) pairs.
//
// Replaces radix_sort_particles_morton_index (src/linear_octree.c:216-326).
// Any stable sort by the full key gives the same order as the reference's
// 9-bit LSD passes, so this sort uses 8-bit digits: per pass
//   1. k_radix_count  -- per-tile digit histograms (4096 elements per tile);
//   2. k_radix_scan_rows -- one CTA per digit: digit base (per-digit totals
//      gathered by the count kernel) plus the scan of that digit's tile
//      counts over the tiles that hold elements;
//   3. k_radix_scatter -- stable in-tile ranks from warp match (each warp
//      owns 512 consecutive elements, 16 rounds of 32, ranked in index
//      order) and scatter to the scanned offsets.
// The element count is read from device memory, so a sort sits inside a
// CUDA graph even when the count is produced on the device (tree nodes).
// HBM-bound: a pass reads 8+4 bytes per element twice and writes them once.
#include "gs_internal.h"
#include "gs_radix.h"

namespace gs {

constexpr int RX_THREADS = 256;
constexpr int RX_ITEMS = 16;
constexpr int RX_TILE = RX_THREADS * RX_ITEMS;   // 4096
constexpr int RX_WARPS = RX_THREADS / 32;

__global__ void __launch_bounds__(RX_THREADS)
k_radix_count(const uint64_t *__restrict__ keys, const int *__restrict__ d_n, int shift, int tiles,
              unsigned *__restrict__ counts, unsigned *__restrict__ totals)
{
    __shared__ unsigned hist[256];
    const int n = *d_n;
    const int base = blockIdx.x * RX_TILE;
    if (base >= n) return;   // block-uniform: tiles past the elements are never read
    hist[threadIdx.x] = 0;
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < RX_ITEMS; ++k) {
        const int e = base + k * RX_THREADS + threadIdx.x;
        if (e < n) atomicAdd(&hist[(unsigned)(keys[e] >> shift) & 255u], 1u);
    }
    __syncthreads();
    const unsigned h = hist[threadIdx.x];
    counts[threadIdx.x * tiles + blockIdx.x] = h;
    if (h) atomicAdd(&totals[threadIdx.x], h);
}

// Output offset of every (digit, tile): the elements of all smaller digits
// (from the per-digit totals) plus those of the same digit in earlier
// tiles.  One CTA per digit scans its row over the tiles holding elements.
__global__ void __launch_bounds__(256)
k_radix_scan_rows(unsigned *__restrict__ counts, const unsigned *__restrict__ totals,
                  const int *__restrict__ d_n, int tiles)
{
    __shared__ unsigned wsum[8];
    const int d = blockIdx.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
    unsigned v = t < d ? totals[t] : 0u;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) wsum[warp] = v;
    __syncthreads();
    unsigned run = 0;
    for (int w = 0; w < 8; ++w) run += wsum[w];
    __syncthreads();
    const int used = (*d_n + RX_TILE - 1) / RX_TILE;
    unsigned *row = counts + (size_t)d * tiles;
    for (int c0 = 0; c0 < used; c0 += 256) {
        const int i = c0 + t;
        const unsigned c = i < used ? row[i] : 0u;
        unsigned incl = c;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        unsigned before = 0, chunk = 0;
        for (int w = 0; w < 8; ++w) {
            const unsigned ws = wsum[w];
            if (w < warp) before += ws;
            chunk += ws;
        }
        if (i < used) row[i] = run + before + incl - c;
        run += chunk;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(RX_THREADS)
k_radix_scatter(const uint64_t *__restrict__ keys_in, const int *__restrict__ vals_in,
                uint64_t *__restrict__ keys_out, int *__restrict__ vals_out,
                const int *__restrict__ d_n, int shift, int tiles,
                const unsigned *__restrict__ offsets)
{
    __shared__ unsigned whist[RX_WARPS][256];
    __shared__ unsigned tile_off[256];
    const int n = *d_n;
    if ((int)blockIdx.x * RX_TILE >= n) return;   // block-uniform
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    for (int d = threadIdx.x; d < RX_WARPS * 256; d += RX_THREADS) (&whist[0][0])[d] = 0u;
    tile_off[threadIdx.x] = offsets[threadIdx.x * tiles + blockIdx.x];
    __syncthreads();

    const int wbase = blockIdx.x * RX_TILE + warp * (RX_ITEMS * 32);
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
    // exclusive prefix over warps, per digit (thread t owns digit t)
    {
        unsigned run = 0;
        for (int w = 0; w < RX_WARPS; ++w) {
            const unsigned c = whist[w][threadIdx.x];
            whist[w][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RX_ITEMS; ++r) {
        const int e = wbase + r * 32 + lane;
        if (e < n) {
            const unsigned d = dig[r];
            const unsigned dst = tile_off[d] + whist[warp][d] + rank[r];
            keys_out[dst] = key[r];
            vals_out[dst] = val[r];
        }
    }
}

ErrorStatus RadixSorter::reserve(int cap)
{
    if (cap <= capacity_) return ok();
    capacity_ = cap;
    tiles_ = (cap + RX_TILE - 1) / RX_TILE;
    GS_TRY(counts_.reserve((size_t)256 * tiles_ * sizeof(unsigned)));
    GS_TRY(totals_.reserve((size_t)8 * 256 * sizeof(unsigned)));
    GS_TRY(tmp_keys_.reserve((size_t)cap * sizeof(uint64_t)));
    GS_TRY(tmp_vals_.reserve((size_t)cap * sizeof(int)));
    return ok();
}

ErrorStatus RadixSorter::sort(uint64_t *keys, int *vals, const int *d_n, int key_bits,
                              cudaStream_t s)
{
    int passes = (key_bits + 7) / 8;
    if (passes & 1) ++passes;   // even: the result lands back in keys / vals
    uint64_t *kin = keys, *kout = tmp_keys_.as<uint64_t>();
    int *vin = vals, *vout = tmp_vals_.as<int>();
    if (passes > 8) return GS_RAISE(GRAV_VALUE_ERROR, "radix sort keys wider than 64 bits");
    GS_CUDA(cudaMemsetAsync(totals_.p, 0, (size_t)passes * 256 * sizeof(unsigned), s));
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        unsigned *tot = totals_.as<unsigned>() + 256 * p;
        k_radix_count<<<tiles_, RX_THREADS, 0, s>>>(kin, d_n, shift, tiles_, counts_.as<unsigned>(),
                                                    tot);
        k_radix_scan_rows<<<256, 256, 0, s>>>(counts_.as<unsigned>(), tot, d_n, tiles_);
        k_radix_scatter<<<tiles_, RX_THREADS, 0, s>>>(kin, vin, kout, vout, d_n, shift, tiles_,
                                                      counts_.as<unsigned>());
        GS_CUDA(cudaGetLastError());
        uint64_t *tk = kin;
        kin = kout;
        kout = tk;
        int *tv = vin;
        vin = vout;
        vout = tv;
    }
    return ok();
}

}  // namespace gs

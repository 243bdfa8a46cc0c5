// k_octree.cu -- GPU construction of grav_sim's linear octree.
//
// Replaces construct_octree and its helpers (src/linear_octree.c:113-962).
// Results equal the reference's: bounding box, Morton keys, sorted order,
// node numbering and topology bit for bit; internal-node mass and centre of
// mass bit for bit (FP64, reference summation order, no FMA contraction).
//
//   bounding box   k_bbox_partial + k_bbox_final: exact FP64 min/max.
//   Morton keys    k_morton: (x - c)/w + 0.5 in FP64, truncation to int64,
//                  21-bit mask (a coordinate at the box maximum wraps to 0,
//                  as in the reference), bit interleave.
//   sort           RadixSorter (stable LSD, 8-bit digits, one sweep per digit) of (key, id).
//   topology       level-synchronous: k_tree_expand(d) splits every internal
//                  node of depth d into its non-empty octants (binary search
//                  on the sorted keys), appending children to an unordered
//                  node list; a child is internal when it holds more than
//                  leaf_max particles and is above depth 21.
//   numbering      the reference numbers nodes in creation order: all
//                  children of a node get consecutive ids when the node is
//                  expanded, and nodes are expanded in depth-first pre-order.
//                  Pre-order of internal nodes is the order of (first
//                  particle, depth), so internal nodes are radix-sorted by
//                  that key and an exclusive scan of their child counts gives
//                  each one's first-child id; a node's id is then its
//                  parent's first-child id plus its octant rank.
//   multipoles     bottom-up in one launch (arrival counters): an internal
//                  node adds, child by child in octant order, the particles
//                  of leaf children (sorted order) and the running sums of
//                  internal children -- the reference's order (:652-735).
//                  Leaves keep mass 0 and centre of mass 0 in compat mode
//                  (the reference's behaviour); otherwise they get their own
//                  sums.  The same kernels write the walk's node records and,
//                  for the quadrupole walks, FP32 quadrupoles.
// Every count the kernels need is read from device memory, so a whole build
// is graph-capturable.  Node-capacity overflow sets ST_TREE_OVERFLOW, which
// stays set until the host reports it; the kernels after the expansion then do
// no work (tree_failed / tree_nodes).
#include "gs_octree.h"
#include "gs_ptx.cuh"

#include <cstdio>

namespace gs {

constexpr int OT_THREADS = 256;
constexpr int BBOX_BLOCKS = 512;
constexpr int SCAN_TILE = 4096;

__device__ __forceinline__ double dmin(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ double dmax(double a, double b) { return fmax(a, b); }

__global__ void __launch_bounds__(OT_THREADS)
k_bbox_partial(const double *__restrict__ x, int n, double *__restrict__ part)
{
    __shared__ double s[6][OT_THREADS];
    double lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = x[k];
        hi[k] = x[k];
    }
    for (int i = blockIdx.x * OT_THREADS + threadIdx.x; i < n; i += gridDim.x * OT_THREADS) {
        for (int k = 0; k < 3; ++k) {
            const double q = x[3 * i + k];
            lo[k] = dmin(lo[k], q);
            hi[k] = dmax(hi[k], q);
        }
    }
    for (int k = 0; k < 3; ++k) {
        s[k][threadIdx.x] = lo[k];
        s[3 + k][threadIdx.x] = hi[k];
    }
    __syncthreads();
    for (int w = OT_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            for (int k = 0; k < 3; ++k) {
                s[k][threadIdx.x] = dmin(s[k][threadIdx.x], s[k][threadIdx.x + w]);
                s[3 + k][threadIdx.x] = dmax(s[3 + k][threadIdx.x], s[3 + k][threadIdx.x + w]);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 6) part[blockIdx.x * 6 + threadIdx.x] = s[threadIdx.x][0];
}

// src/linear_octree.c:138-145 (and :856-867 when a box is given)
// One CTA of OT_THREADS threads: min / max are exact in any order, so the
// block partials are reduced as a tree.
__global__ void __launch_bounds__(OT_THREADS)
k_bbox_final(const double *__restrict__ part, int blocks, double ocx, double ocy, double ocz,
             double owidth, double *__restrict__ frame)
{
    __shared__ double s[6][OT_THREADS];
    double lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = part[k];
        hi[k] = part[3 + k];
    }
    for (int b = threadIdx.x; b < blocks; b += OT_THREADS)
        for (int k = 0; k < 3; ++k) {
            lo[k] = dmin(lo[k], part[6 * b + k]);
            hi[k] = dmax(hi[k], part[6 * b + 3 + k]);
        }
    for (int k = 0; k < 3; ++k) {
        s[k][threadIdx.x] = lo[k];
        s[3 + k][threadIdx.x] = hi[k];
    }
    __syncthreads();
    for (int w2 = OT_THREADS / 2; w2 > 0; w2 >>= 1) {
        if (threadIdx.x < w2) {
            for (int k = 0; k < 3; ++k) {
                s[k][threadIdx.x] = dmin(s[k][threadIdx.x], s[k][threadIdx.x + w2]);
                s[3 + k][threadIdx.x] = dmax(s[3 + k][threadIdx.x], s[3 + k][threadIdx.x + w2]);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    for (int k = 0; k < 3; ++k) {
        lo[k] = s[k][0];
        hi[k] = s[3 + k][0];
    }
    double c[3], w;
    if (owidth > 0.0) {
        c[0] = ocx;
        c[1] = ocy;
        c[2] = ocz;
        w = owidth;
    } else {
        for (int k = 0; k < 3; ++k) c[k] = __ddiv_rn(__dadd_rn(hi[k], lo[k]), 2.0);
        w = dmax(dmax(__dsub_rn(hi[0], lo[0]), __dsub_rn(hi[1], lo[1])), __dsub_rn(hi[2], lo[2]));
    }
    frame[0] = c[0];
    frame[1] = c[1];
    frame[2] = c[2];
    frame[3] = w;
    frame[4] = __dmul_rn(w, 2.0);
    // the width's double-word reciprocal for div_by_width: zh = RN(1/w) and
    // zl = RN(1/w - zh), where 1 - zh w is exact (zh is correctly rounded)
    const double zh = __ddiv_rn(1.0, w);
    frame[5] = zh;
    frame[6] = __ddiv_rn(__fma_rn(-zh, w, 1.0), w);
    const double aw = fabs(w);
    frame[7] = (aw >= 0x1p-100 && aw <= 0x1p+100) ? 1.0 : 0.0;
}

// RN(x / w) for the box width w = frame[3] without a division, from the
// double-word reciprocal (frame[5], frame[6]) that k_bbox_final stored:
// q = RN(x zh + RN(x zl)) is within an ulp of x / w (Brisebarre, Muller and
// Raina, IEEE Trans. Computers 53(8), 2004), and the exact remainder
// r = x - q w corrects it to RN(q + r zh) = RN(x / w) (Markstein, IBM J.
// Res. Dev. 34(1), 1990).  The remainder is exact while its last bit stays
// above the subnormal range: |w| in [2^-100, 2^100] (frame[7]) and |x| in
// [2^-900, 2^900]; other operands (zeros, subnormals, infinities, NaN)
// take the division itself.  Checked against __ddiv_rn bit for bit by
// gsgpu_width_division_selftest.
__device__ __forceinline__ double div_by_width(double x, const double *__restrict__ frame)
{
    const double ax = fabs(x);
    if (frame[7] == 0.0 || !(ax >= 0x1p-900 && ax <= 0x1p+900)) return __ddiv_rn(x, frame[3]);
    const double q = __fma_rn(x, frame[5], __dmul_rn(x, frame[6]));
    const double r = __fma_rn(-q, frame[3], x);
    return __fma_rn(r, frame[5], q);
}

// 21 low bits of v spread to every third bit (magic-number interleave).
__device__ __forceinline__ uint64_t spread3(uint64_t v)
{
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x001f00000000ffffull;
    v = (v | (v << 16)) & 0x001f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// src/linear_octree.c:159-202
__global__ void k_morton(const double *__restrict__ x, int n, const double *__restrict__ frame,
                         uint64_t *__restrict__ keys, int *__restrict__ sidx,
                         unsigned char *__restrict__ misplaced)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t k = 0;
    bool out = false;   // a coordinate outside [0, 2^21) is masked: the key cell is elsewhere
    for (int d = 0; d < 3; ++d) {
        const double u = __dadd_rn(div_by_width(__dsub_rn(x[3 * i + d], frame[d]), frame), 0.5);
        const long long q = __double2ll_rz(__dmul_rn(u, 2097152.0));
        out = out || q < 0 || q > 0x1fffffll;
        k |= spread3((uint64_t)q) << d;
    }
    keys[i] = k;
    sidx[i] = i;
    misplaced[i] = out ? 1 : 0;
}

__global__ void k_tree_init(int *__restrict__ ctr, int n, int *__restrict__ nd_start,
                            int *__restrict__ nd_count, int *__restrict__ nd_depth,
                            int *__restrict__ nd_parent, int *__restrict__ nd_rank,
                            int *__restrict__ nd_int, int *__restrict__ in_node)
{
    if (threadIdx.x != 0) return;
    ctr[CTR_NODES] = 1;
    ctr[CTR_INTERNAL] = 1;
    ctr[CTR_N] = n;
    ctr[CTR_LVL + 0] = 0;
    ctr[CTR_LVL + 1] = 1;
    nd_start[0] = 0;
    nd_count[0] = n;
    nd_depth[0] = 0;
    nd_parent[0] = -1;
    nd_rank[0] = 0;
    nd_int[0] = 0;
    in_node[0] = 0;
}

// First index in [lo, hi) whose octant digit at `shift` exceeds o.
__device__ __forceinline__ int octant_end(const uint64_t *__restrict__ keys, int lo, int hi,
                                          int shift, int o)
{
    while (lo < hi) {
        const int mid = lo + ((hi - lo) >> 1);
        const int dig = (int)((keys[mid] >> shift) & 7ull);
        if (dig <= o)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// src/linear_octree.c:342-576 for all internal nodes of depth d at once.
// Levels with few nodes (the top of the tree, where a node's binary
// searches are long) use eight lanes per node, one per octant: each finds
// where its octant ends by its own binary search over the node's sorted
// keys (the searches are independent: the keys of a node are sorted by
// their octant digit), the eight ends are combined by shuffles within the
// 8-lane group, and each lane writes its own child.  Levels with many nodes
// use one thread per node.  Node ids come from an atomic counter; the
// reference's numbering is recovered later by k_tree_number.
constexpr int EXPAND_WIDE_NODES = 16384;
__global__ void __launch_bounds__(OT_THREADS)
k_tree_expand(int d, int leaf_max, int cap, const uint64_t *__restrict__ keys, int *__restrict__ ctr,
              int *__restrict__ nd_start, int *__restrict__ nd_count, int *__restrict__ nd_depth,
              int *__restrict__ nd_parent, int *__restrict__ nd_rank, int *__restrict__ nd_int,
              int *__restrict__ in_node, int *__restrict__ in_nchild)
{
    if (tree_failed(ctr)) return;   // an earlier level overflowed
    const int lo = ctr[CTR_LVL + d];
    const int hi = ctr[CTR_LVL + d + 1];
    const int cd = d + 1;
    const int shift = 3 * (OCT_MAX_LEVEL - cd);
    if (hi - lo > EXPAND_WIDE_NODES) {
        // many nodes (deep levels, few particles each): one thread per node,
        // its eight searches over shrinking ranges
        for (int ii = lo + blockIdx.x * OT_THREADS + threadIdx.x; ii < hi;
             ii += gridDim.x * OT_THREADS) {
            const int q = in_node[ii];
            const int s = nd_start[q];
            const int e = s + nd_count[q];
            int ends[8];
            int nch = 0;
            int prev = s;
            for (int o = 0; o < 8; ++o) {
                ends[o] = octant_end(keys, prev, e, shift, o);
                if (ends[o] > prev) ++nch;
                prev = ends[o];
            }
            const int base = atomicAdd(&ctr[CTR_NODES], nch);
            if (base + nch > cap) {
                atomicOr((unsigned *)&ctr[CTR_STATUS], ST_TREE_OVERFLOW);
                in_nchild[ii] = 0;
                continue;
            }
            int r = 0;
            prev = s;
            for (int o = 0; o < 8; ++o) {
                const int cnt = ends[o] - prev;
                if (cnt > 0) {
                    const int c = base + r;
                    nd_start[c] = prev;
                    nd_count[c] = cnt;
                    nd_depth[c] = cd;
                    nd_parent[c] = ii;
                    nd_rank[c] = r;
                    int slot = -1;
                    if (cnt > leaf_max && cd < OCT_MAX_LEVEL) {
                        slot = atomicAdd(&ctr[CTR_INTERNAL], 1);
                        if (slot >= cap) {
                            atomicOr((unsigned *)&ctr[CTR_STATUS], ST_TREE_OVERFLOW);
                            slot = -1;
                        } else {
                            in_node[slot] = c;
                        }
                    }
                    nd_int[c] = slot;
                    ++r;
                }
                prev = ends[o];
            }
            in_nchild[ii] = nch;
        }
        return;
    }
    const int lane = threadIdx.x & 31;
    const int o = lane & 7;
    const int g0 = lane & ~7;   // first lane of this node's group
    for (int wt = blockIdx.x * OT_THREADS + (threadIdx.x & ~31);; wt += gridDim.x * OT_THREADS) {
        if (lo + (wt >> 3) >= hi) break;   // warp-uniform
        const int ii = lo + ((wt + lane) >> 3);
        const bool act = ii < hi;
        int s = 0, e = 0;
        if (act) {
            const int q = in_node[ii];
            s = nd_start[q];
            e = s + nd_count[q];
        }
        const int endo = act ? octant_end(keys, s, e, shift, o) : 0;
        const int up = __shfl_up_sync(0xffffffffu, endo, 1, 8);
        const int prev = (o == 0) ? s : up;
        const int cnt = act ? endo - prev : 0;
        const unsigned m8 = (__ballot_sync(0xffffffffu, cnt > 0) >> g0) & 0xffu;
        const int nch = __popc(m8);
        const int rank = __popc(m8 & ((1u << o) - 1u));
        int base = 0;
        if (act && o == 0) base = atomicAdd(&ctr[CTR_NODES], nch);
        base = __shfl_sync(0xffffffffu, base, g0);
        if (!act) continue;
        if (base + nch > cap) {
            if (o == 0) {
                atomicOr((unsigned *)&ctr[CTR_STATUS], ST_TREE_OVERFLOW);
                in_nchild[ii] = 0;
            }
            continue;
        }
        if (cnt > 0) {
            const int c = base + rank;
            nd_start[c] = prev;
            nd_count[c] = cnt;
            nd_depth[c] = cd;
            nd_parent[c] = ii;
            nd_rank[c] = rank;
            int slot = -1;
            if (cnt > leaf_max && cd < OCT_MAX_LEVEL) {
                slot = atomicAdd(&ctr[CTR_INTERNAL], 1);
                if (slot >= cap) {
                    atomicOr((unsigned *)&ctr[CTR_STATUS], ST_TREE_OVERFLOW);
                    slot = -1;
                } else {
                    in_node[slot] = c;
                }
            }
            nd_int[c] = slot;
        }
        if (o == 0) in_nchild[ii] = nch;
    }
}

__global__ void k_tree_mark(int d, int *__restrict__ ctr)
{
    if (threadIdx.x == 0) {
        ctr[CTR_LVL + d + 2] = ctr[CTR_INTERNAL];
        ctr[CTR_SAFE_INTERNAL] = tree_failed(ctr) ? 0 : ctr[CTR_INTERNAL];
    }
}

// Sort key of an internal node: pre-order = (first particle, depth).
__global__ void k_internal_keys(const int *__restrict__ ctr, const int *__restrict__ in_node,
                                const int *__restrict__ nd_start, const int *__restrict__ nd_depth,
                                uint64_t *__restrict__ in_key, int *__restrict__ in_order,
                                int *__restrict__ in_arrive)
{
    const int ni = ctr[CTR_SAFE_INTERNAL];
    for (int ii = blockIdx.x * blockDim.x + threadIdx.x; ii < ni; ii += gridDim.x * blockDim.x) {
        const int q = in_node[ii];
        in_key[ii] = ((uint64_t)nd_start[q] << 5) | (uint64_t)nd_depth[q];
        in_order[ii] = ii;
        in_arrive[ii] = 0;
    }
}

// Tile sums of child counts in pre-order.
__global__ void __launch_bounds__(OT_THREADS)
k_fc_tile_sums(const int *__restrict__ ctr, const int *__restrict__ in_order,
               const int *__restrict__ in_nchild, unsigned *__restrict__ tile_sum)
{
    __shared__ unsigned red[OT_THREADS];
    const int ni = ctr[CTR_SAFE_INTERNAL];
    const int base = blockIdx.x * SCAN_TILE;
    unsigned s = 0;
    for (int k = threadIdx.x; k < SCAN_TILE; k += OT_THREADS) {
        const int e = base + k;
        if (e < ni) s += (unsigned)in_nchild[in_order[e]];
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = OT_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(1024) k_scan_small(unsigned *__restrict__ v, int len)
{
    __shared__ unsigned part[1024];
    const int per = (len + 1023) / 1024;
    const int b = threadIdx.x * per;
    const int e = min(len, b + per);
    unsigned s = 0;
    for (int i = b; i < e; ++i) s += v[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const unsigned t = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += t;
        __syncthreads();
    }
    unsigned run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
    for (int i = b; i < e; ++i) {
        const unsigned c = v[i];
        v[i] = run;
        run += c;
    }
}

// First-child id of each internal node: 1 + exclusive scan in pre-order.
__global__ void __launch_bounds__(OT_THREADS)
k_fc_apply(const int *__restrict__ ctr, const int *__restrict__ in_order,
           const int *__restrict__ in_nchild, const unsigned *__restrict__ tile_off,
           int *__restrict__ in_fc)
{
    constexpr int PER = SCAN_TILE / OT_THREADS;   // 16 consecutive per thread
    __shared__ unsigned part[OT_THREADS];
    const int ni = ctr[CTR_SAFE_INTERNAL];
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * PER;
    unsigned v[PER];
    unsigned s = 0;
    for (int k = 0; k < PER; ++k) {
        const int e = base + k;
        v[k] = e < ni ? (unsigned)in_nchild[in_order[e]] : 0u;
        s += v[k];
    }
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < OT_THREADS; off <<= 1) {
        const unsigned t = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += t;
        __syncthreads();
    }
    unsigned run = tile_off[blockIdx.x] + (threadIdx.x ? part[threadIdx.x - 1] : 0u);
    for (int k = 0; k < PER; ++k) {
        const int e = base + k;
        if (e < ni) in_fc[in_order[e]] = 1 + (int)run;
        run += v[k];
    }
}

// Final node arrays by id.
__global__ void k_tree_number(const int *__restrict__ ctr, int compat,
                              const int *__restrict__ nd_start, const int *__restrict__ nd_count,
                              const int *__restrict__ nd_depth, const int *__restrict__ nd_parent,
                              const int *__restrict__ nd_rank, const int *__restrict__ nd_int,
                              const int *__restrict__ in_nchild, const int *__restrict__ in_fc,
                              int *__restrict__ in_id, int *__restrict__ t_np,
                              int *__restrict__ t_nc, int *__restrict__ t_fp,
                              int *__restrict__ t_fc, int *__restrict__ t_depth,
                              int *__restrict__ t_int, double *__restrict__ t_mass,
                              double *__restrict__ t_com)
{
    const int nn = tree_nodes(ctr);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nn; q += gridDim.x * blockDim.x) {
        const int id = (q == 0) ? 0 : in_fc[nd_parent[q]] + nd_rank[q];
        t_np[id] = nd_count[q];
        t_fp[id] = nd_start[q];
        t_depth[id] = nd_depth[q];
        const int ii = nd_int[q];
        t_int[id] = ii;
        if (ii >= 0) {
            t_nc[id] = in_nchild[ii];
            t_fc[id] = in_fc[ii];
            in_id[ii] = id;
        } else {
            t_nc[id] = 0;
            t_fc[id] = -1;
            if (compat) {
                t_mass[id] = 0.0;
                t_com[3 * id + 0] = 0.0;
                t_com[3 * id + 1] = 0.0;
                t_com[3 * id + 2] = 0.0;
            }
        }
    }
}

// Parent id of every node and the leaf of every sorted particle (used by
// the learned method's features).
__global__ void k_tree_links(const int *__restrict__ ctr, const int *__restrict__ nd_start,
                             const int *__restrict__ nd_count, const int *__restrict__ nd_parent,
                             const int *__restrict__ nd_rank, const int *__restrict__ nd_int,
                             const int *__restrict__ in_node, const int *__restrict__ in_fc,
                             int *__restrict__ t_parent, int *__restrict__ leaf_of)
{
    const int nn = tree_nodes(ctr);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nn; q += gridDim.x * blockDim.x) {
        int id = 0, parent = -1;
        if (q != 0) {
            id = in_fc[nd_parent[q]] + nd_rank[q];
            const int pq = in_node[nd_parent[q]];
            parent = (pq == 0) ? 0 : in_fc[nd_parent[pq]] + nd_rank[pq];
        }
        t_parent[id] = parent;
        if (nd_int[q] < 0)
            for (int p = nd_start[q]; p < nd_start[q] + nd_count[q]; ++p) leaf_of[p] = id;
    }
}

// Running sums of the particles of one leaf, sorted order (reference :667-674).
// Mass and mass-weighted coordinate sums of sorted particles [first,
// first + count) in sorted order (the reference's order), read from the
// sorted (x, y, z, m) copy: contiguous 32-byte records instead of gathers
// through the sorted ids into the caller's arrays; same values, same sums.
__device__ __forceinline__ void add_particles(const double *__restrict__ xm, int first, int count,
                                              double &M, double &S0, double &S1, double &S2)
{
#pragma unroll 4
    for (int p = first; p < first + count; ++p) {
        const double2 a = __ldg(reinterpret_cast<const double2 *>(xm + 4 * (size_t)p));
        const double2 b = __ldg(reinterpret_cast<const double2 *>(xm + 4 * (size_t)p) + 1);
        const double mp = b.y;
        M = __dadd_rn(M, mp);
        S0 = __dadd_rn(S0, __dmul_rn(mp, a.x));
        S1 = __dadd_rn(S1, __dmul_rn(mp, a.y));
        S2 = __dadd_rn(S2, __dmul_rn(mp, b.x));
    }
}

__device__ __forceinline__ void split_df(double v, float &hi, float &lo)
{
    hi = __double2float_rn(v);
    lo = __double2float_rn(__dsub_rn(v, (double)hi));
}

// (cell side)^2 at depth d, box_length / (2 << d), for the group walk's
// opening test.  The divisor is a power of two, so the product with its
// exact reciprocal (built from the exponent bits) equals the quotient.
__device__ __forceinline__ float cell_side2(const double *__restrict__ frame, int depth)
{
    const int e = min(depth, OCT_MAX_LEVEL + 1) + 1;
    const double side = __dmul_rn(frame[4], __longlong_as_double((long long)(1023 - e) << 52));
    return (float)(side * side);
}

// Walk record of a node: centre of mass relative to the frame centre as
// (hi, lo) FP32 pairs, FP32 mass, (cell side)^2.  The same arithmetic for
// every node, whichever kernel computes its multipoles.
__device__ __forceinline__ void write_node_record(int id, double M, double c0, double c1, double c2,
                                                  int depth, const double *__restrict__ frame,
                                                  float4 *na, float4 *nb, float h[3], float l[3])
{
    split_df(__dsub_rn(c0, frame[0]), h[0], l[0]);
    split_df(__dsub_rn(c1, frame[1]), h[1], l[1]);
    split_df(__dsub_rn(c2, frame[2]), h[2], l[2]);
    na[id] = make_float4(h[0], h[1], h[2], (float)M);
    nb[id] = make_float4(l[0], l[1], l[2], cell_side2(frame, depth));
}

// m (3 d d^T - |d|^2 I) added to the packed quadrupole (xx, xy, xz, yy, yz, zz).
__device__ __forceinline__ void add_quad(float Q[6], float mp, float d0, float d1, float d2)
{
    const float r2 = d0 * d0 + d1 * d1 + d2 * d2;
    const float m3 = 3.0f * mp;
    Q[0] += mp * (3.0f * d0 * d0 - r2);
    Q[1] += m3 * d0 * d1;
    Q[2] += m3 * d0 * d2;
    Q[3] += mp * (3.0f * d1 * d1 - r2);
    Q[4] += m3 * d1 * d2;
    Q[5] += mp * (3.0f * d2 * d2 - r2);
}

__device__ __forceinline__ void store_quad(float4 *nq, int id, const float Q[6])
{
    nq[2 * (size_t)id] = make_float4(Q[0], Q[1], Q[2], Q[3]);
    nq[2 * (size_t)id + 1] = make_float4(Q[4], Q[5], 0.0f, 0.0f);
}

// Offset of a (hi, lo) FP32 pair point from a (hi, lo) centre, in FP32:
// the hi parts of points in one cell are close, so their difference is
// exact, and the lo parts carry the rest.
__device__ __forceinline__ float df_offset(float ph, float pl, float ch, float cl)
{
    return (ph - ch) + (pl - cl);
}

struct MultipoleArgs {
    const double *xm;   // sorted (x, y, z, m) records
    const int *sidx, *in_node, *nd_parent, *in_id, *in_fc, *in_nchild;
    const int *t_np, *t_nc, *t_fp, *t_int, *t_depth;
    const double *frame;
    int *in_arrive;
    double *in_sum, *t_mass, *t_com;
    float4 *na, *nb, *nq;   // nq null: no quadrupoles
};

// Multipoles of internal node ii from its children (reference :652-735): mass
// and the mass-weighted coordinate sums in child order, the centre of mass by
// division, its walk record, and, when nq is not null, the quadrupole from the
// children's by the parallel-axis shift Q = sum_c [Q_c + M_c (3 s s^T - |s|^2 I)],
// s = com_c - com, in FP32 from the children's walk records (FP64 runs at 1/64
// of the FP32 rate here, and the walk uses FP32 quadrupoles).  Children's
// values written by other threads of the same launch are read through L2
// (__ldcg), after the fence that follows the arrival counter.
//
// A node is computed by the four lanes of a group: lane j keeps one of the
// four ordered sums (j = 0 the mass, j = 1..3 the sums of m x, m y, m z), so
// a particle costs one FP64 multiply and one add for all four sums (lane 0
// multiplies the mass by 1.0, which is exact: its sum is the plain mass sum),
// and the three quotients are one division.  An FP64 warp instruction costs
// the pipe a whole warp's time however few lanes it carries, and near the
// root a single group climbs alone: this cuts the FP64 instructions on that
// path from 7 to 2 per particle.  Each sum sees the same operands in the same
// order as a one-thread loop would, so the values are the same bit for bit.
__device__ void multipole_node4(int ii, int j, unsigned gmask, const MultipoleArgs &A)
{
    const int fc = A.in_fc[ii];
    const int end = fc + A.in_nchild[ii];
    double acc = 0.0;
    for (int c = fc; c < end; ++c) {
        if (A.t_nc[c] > 0) {
            acc = __dadd_rn(acc, __ldcg(A.in_sum + 4 * (size_t)A.t_int[c] + j));
        } else {
            const int p1 = A.t_fp[c] + A.t_np[c];
#pragma unroll 4
            for (int p = A.t_fp[c]; p < p1; ++p) {
                const double *r = A.xm + 4 * (size_t)p;
                const double mp = __ldg(r + 3);
                const double xv = j == 0 ? 1.0 : __ldg(r + j - 1);
                acc = __dadd_rn(acc, __dmul_rn(mp, xv));
            }
        }
    }
    A.in_sum[4 * (size_t)ii + j] = acc;
    const double M = __shfl_sync(gmask, acc, 0, 4);
    const double cj = __ddiv_rn(acc, M);   // lanes 1..3: coordinate j - 1 of the centre
    const int id = A.in_id[ii];
    float hj = 0.0f, lj = 0.0f;
    if (j == 0) {
        A.t_mass[id] = M;
    } else {
        A.t_com[3 * id + j - 1] = cj;
        split_df(__dsub_rn(cj, A.frame[j - 1]), hj, lj);
    }
    float h[3], l[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        h[k] = __shfl_sync(gmask, hj, k + 1, 4);
        l[k] = __shfl_sync(gmask, lj, k + 1, 4);
    }
    if (j == 0) {
        A.na[id] = make_float4(h[0], h[1], h[2], (float)M);
        A.nb[id] = make_float4(l[0], l[1], l[2], cell_side2(A.frame, A.t_depth[id]));
    }
    if (A.nq) {
        // every lane of the group forms the same sums; lane 0 stores them
        float Q[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int c = fc; c < end; ++c) {
            const float4 ca = __ldcg(A.na + c), cb = __ldcg(A.nb + c);
            const float4 qa = __ldcg(A.nq + 2 * (size_t)c), qb = __ldcg(A.nq + 2 * (size_t)c + 1);
            add_quad(Q, ca.w, df_offset(ca.x, cb.x, h[0], l[0]), df_offset(ca.y, cb.y, h[1], l[1]),
                     df_offset(ca.z, cb.z, h[2], l[2]));
            Q[0] += qa.x;
            Q[1] += qa.y;
            Q[2] += qa.z;
            Q[3] += qa.w;
            Q[4] += qb.x;
            Q[5] += qb.y;
        }
        if (j == 0) store_quad(A.nq, id, Q);
    }
}

// All internal nodes in one launch, bottom-up.  A group of four lanes starts
// at each internal node none of whose children is internal, computes it, and
// climbs: it counts itself in the parent's arrival counter, and the group that
// completes the count (the last of the parent's internal children to finish)
// computes the parent.  Nothing waits: a group that is not last stops.  Every
// node is computed once, by the same arithmetic in the same child order as a
// level-by-level pass, so the sums are identical to it.  Every decision below
// is the same for the four lanes of a group (they share the node), so the
// group's shuffles and barriers see all four.
__global__ void __launch_bounds__(OT_THREADS) k_multipole_up(const int *__restrict__ ctr,
                                                             MultipoleArgs A)
{
    const int ni = ctr[CTR_SAFE_INTERNAL];
    const int j = threadIdx.x & 3;
    const unsigned gmask = 0xFu << ((threadIdx.x & 31) & ~3);
    const int groups = (gridDim.x * blockDim.x) >> 2;
    for (int i0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 2; i0 < ni; i0 += groups) {
        const int fc0 = A.in_fc[i0];
        const int nch0 = A.in_nchild[i0];
        bool bottom = true;
        for (int c = fc0; c < fc0 + nch0; ++c) bottom = bottom && A.t_nc[c] == 0;
        if (!bottom) continue;
        int ii = i0;
        for (;;) {
            multipole_node4(ii, j, gmask, A);
            const int p = A.nd_parent[A.in_node[ii]];
            if (p < 0) break;
            const int fc = A.in_fc[p];
            const int nch = A.in_nchild[p];
            int internal = 0;
            for (int c = fc; c < fc + nch; ++c) internal += A.t_nc[c] > 0 ? 1 : 0;
            // each lane's writes are visible before lane 0 counts the group in
            __threadfence();
            __syncwarp(gmask);
            int arrived = 0;
            if (j == 0) arrived = atomicAdd(&A.in_arrive[p], 1);
            arrived = __shfl_sync(gmask, arrived, 0, 4);
            if (arrived != internal - 1) break;
            __threadfence();
            ii = p;
        }
    }
}

// Leaves with their own mass and centre of mass (non-compat trees), their walk
// records, and, when nq is not null, their quadrupole sum_p m (3 d d^T - |d|^2 I)
// about the centre of mass, from the particles' (hi, lo) FP32 pairs.
__global__ void k_leaf_multipoles(const int *__restrict__ ctr, MultipoleArgs A,
                                  const float4 *__restrict__ pa, const float4 *__restrict__ pb)
{
    const int nn = tree_nodes(ctr);
    for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < nn; id += gridDim.x * blockDim.x) {
        if (A.t_nc[id] > 0) continue;
        const int fp = A.t_fp[id], np = A.t_np[id];
        double M = 0.0, S0 = 0.0, S1 = 0.0, S2 = 0.0;
        add_particles(A.xm, fp, np, M, S0, S1, S2);
        const double c0 = __ddiv_rn(S0, M), c1 = __ddiv_rn(S1, M), c2 = __ddiv_rn(S2, M);
        A.t_mass[id] = M;
        A.t_com[3 * id + 0] = c0;
        A.t_com[3 * id + 1] = c1;
        A.t_com[3 * id + 2] = c2;
        float h[3], l[3];
        write_node_record(id, M, c0, c1, c2, A.t_depth[id], A.frame, A.na, A.nb, h, l);
        if (A.nq) {
            float Q[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
            for (int p = fp; p < fp + np; ++p) {
                const float4 a = pa[p], b = pb[p];
                add_quad(Q, a.w, df_offset(a.x, b.x, h[0], l[0]), df_offset(a.y, b.y, h[1], l[1]),
                         df_offset(a.z, b.z, h[2], l[2]));
            }
            store_quad(A.nq, id, Q);
        }
    }
}

// Walk arrays of every node: (first child, children, first particle,
// particles), the membership key, and the records of the nodes whose
// multipoles the kernels above did not compute -- the zero-mass leaves of a
// compat tree.
__global__ void k_walk_nodes(const int *__restrict__ ctr, int compat, const double *__restrict__ frame,
                             const uint64_t *__restrict__ keys, const int *__restrict__ sidx,
                             const int *__restrict__ t_np, const int *__restrict__ t_nc,
                             const int *__restrict__ t_fp, const int *__restrict__ t_fc,
                             const int *__restrict__ t_depth,
                             const double *__restrict__ t_mass, const double *__restrict__ t_com,
                             float4 *__restrict__ na, float4 *__restrict__ nb, int4 *__restrict__ nc,
                             uint64_t *__restrict__ nkey)
{
    const int nn = tree_nodes(ctr);
    for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < nn; id += gridDim.x * blockDim.x) {
        if (compat && t_nc[id] == 0) {
            float h[3], l[3];
            write_node_record(id, t_mass[id], t_com[3 * id], t_com[3 * id + 1], t_com[3 * id + 2],
                              t_depth[id], frame, na, nb, h, l);
        }
        const int fp = t_fp[id];
        nc[id] = make_int4(t_fc[id], t_nc[id], fp, t_np[id]);
        // the reference's membership test reads keys[sorted_indices[first]]
        // from the sorted key array (src/acceleration_barnes_hut.c:145)
        nkey[id] = compat ? keys[sidx[fp]] : keys[fp];
    }
}

__global__ void k_walk_particles(int n, const double *__restrict__ frame, const double *__restrict__ x,
                                 const double *__restrict__ m, const int *__restrict__ sidx,
                                 float4 *__restrict__ pa, float4 *__restrict__ pb,
                                 double *__restrict__ xm,
                                 const unsigned char *__restrict__ misplaced,
                                 int *__restrict__ mlist)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int id = sidx[p];
    if (misplaced[id]) {   // rare: the count, and the sorted positions of the first ones
        const int at = atomicAdd(&mlist[0], 1);
        if (at < kMisplacedCap) mlist[1 + at] = p;
    }
    double2 *xo = reinterpret_cast<double2 *>(xm + 4 * (size_t)p);
    xo[0] = make_double2(x[3 * id + 0], x[3 * id + 1]);
    xo[1] = make_double2(x[3 * id + 2], m[id]);
    float h0, l0, h1, l1, h2, l2;
    split_df(__dsub_rn(x[3 * id + 0], frame[0]), h0, l0);
    split_df(__dsub_rn(x[3 * id + 1], frame[1]), h1, l1);
    split_df(__dsub_rn(x[3 * id + 2], frame[2]), h2, l2);
    pa[p] = make_float4(h0, h1, h2, (float)m[id]);
    pb[p] = make_float4(l0, l1, l2, 0.0f);
}

// ------------------------------------------------------------------------
ErrorStatus OctreeDevice::setup(int n_, int leaf_max_, bool compat_, bool quad_)
{
    n = n_;
    leaf_max = leaf_max_;
    compat = compat_;
    quad = quad_ && !compat_;
    int cap = 4 * n + 4096;
    if (cap < n) return GS_RAISE(GRAV_VALUE_ERROR, "too many particles for the octree: %d", n);
    cap_nodes = cap;
    const size_t ci = (size_t)cap * sizeof(int);
    GS_TRY(ctr.reserve(CTR_SIZE * sizeof(int)));
    GS_CUDA(cudaMemset(ctr.p, 0, CTR_SIZE * sizeof(int)));   // status word starts clear
    GS_TRY(frame.reserve(8 * sizeof(double)));
    GS_TRY(bbox_part.reserve((size_t)BBOX_BLOCKS * 6 * sizeof(double)));
    GS_TRY(keys.reserve((size_t)n * sizeof(uint64_t)));
    GS_TRY(sidx.reserve((size_t)n * sizeof(int)));
    DBuf *ints[] = {&nd_start, &nd_count, &nd_depth, &nd_parent, &nd_rank, &nd_int, &in_node,
                    &in_nchild, &in_fc, &in_id, &in_order, &t_np, &t_nc, &t_fp, &t_fc, &t_depth,
                    &t_int};
    for (DBuf *b : ints) GS_TRY(b->reserve(ci));
    GS_TRY(in_key.reserve((size_t)cap * sizeof(uint64_t)));
    GS_TRY(scan_tiles.reserve((size_t)((cap + SCAN_TILE - 1) / SCAN_TILE + 1) * sizeof(unsigned)));
    GS_TRY(t_mass.reserve((size_t)cap * sizeof(double)));
    GS_TRY(t_com.reserve((size_t)cap * 3 * sizeof(double)));
    GS_TRY(in_sum.reserve((size_t)cap * 4 * sizeof(double)));
    GS_TRY(in_arrive.reserve(ci));
    GS_TRY(w_na.reserve((size_t)cap * sizeof(float4)));
    GS_TRY(w_nb.reserve((size_t)cap * sizeof(float4)));
    GS_TRY(w_nc.reserve((size_t)cap * sizeof(int4)));
    GS_TRY(w_nkey.reserve((size_t)cap * sizeof(uint64_t)));
    GS_TRY(misplaced.reserve((size_t)n));
    GS_TRY(mlist.reserve((size_t)(1 + kMisplacedCap) * sizeof(int)));
    GS_TRY(w_pa.reserve((size_t)n * sizeof(float4)));
    GS_TRY(w_pb.reserve((size_t)n * sizeof(float4)));
    GS_TRY(xm.reserve((size_t)n * 4 * sizeof(double)));
    GS_TRY(g_list.reserve((size_t)n * sizeof(int2)));
    GS_TRY(g_ctr.reserve(4 * sizeof(int)));
    if (quad) GS_TRY(w_nq.reserve((size_t)cap * 2 * sizeof(float4)));
    if (links) {
        GS_TRY(t_parent.reserve((size_t)cap * sizeof(int)));
        GS_TRY(leaf_of.reserve((size_t)n * sizeof(int)));
    }
    GS_TRY(sorter.reserve(std::max(n, cap)));
    return ok();
}

int OctreeDevice::launches_per_build() const
{
    // bbox 2, morton 1, sort, init 1, levels 2*21, keys 1, sort, fc 3,
    // number 1, multipoles 1 (+1 leaves; quadrupoles in the same launches),
    // walk arrays 2
    return 2 + 1 + RadixSorter::launches(63) + 1 + 42 + 1 +
           RadixSorter::launches(internal_key_bits()) + 3 + 1 +
           1 + (compat ? 0 : 1) + 2 + (links ? 1 : 0);
}

ErrorStatus OctreeDevice::build(const double *d_x, const double *d_m, cudaStream_t s,
                                const double *box_center, double box_width)
{
    const int nb = std::min(BBOX_BLOCKS, std::max(1, (n + OT_THREADS - 1) / OT_THREADS));
    k_bbox_partial<<<nb, OT_THREADS, 0, s>>>(d_x, n, bbox_part.as<double>());
    const bool own_box = box_center && box_width > 0.0;
    k_bbox_final<<<1, OT_THREADS, 0, s>>>(bbox_part.as<double>(), nb, own_box ? box_center[0] : 0.0,
                                  own_box ? box_center[1] : 0.0, own_box ? box_center[2] : 0.0,
                                  own_box ? box_width : -1.0, frame.as<double>());
    const int pb = (n + OT_THREADS - 1) / OT_THREADS;
    if (tm_morton) GS_TRY(tm_morton->begin(s));
    k_morton<<<pb, OT_THREADS, 0, s>>>(d_x, n, frame.as<double>(), keys.as<uint64_t>(),
                                       sidx.as<int>(), misplaced.as<unsigned char>());
    if (tm_morton) GS_TRY(tm_morton->end(s));
    k_tree_init<<<1, 32, 0, s>>>(ctr.as<int>(), n, nd_start.as<int>(), nd_count.as<int>(),
                                 nd_depth.as<int>(), nd_parent.as<int>(), nd_rank.as<int>(),
                                 nd_int.as<int>(), in_node.as<int>());
    GS_CUDA(cudaGetLastError());
    if (tm_sort) GS_TRY(tm_sort->begin(s));
    GS_TRY(sorter.sort(keys.as<uint64_t>(), sidx.as<int>(), ctr.as<int>() + CTR_N, n, 63,
                       reinterpret_cast<unsigned *>(ctr.as<int>() + CTR_STATUS), s));
    if (tm_sort) GS_TRY(tm_sort->end(s));

    const DeviceInfo *dev = nullptr;
    GS_TRY(device_info(&dev));
    // Grid-stride kernels: two CTAs per SM cover the largest levels, and a
    // small grid keeps the launches of the many small levels cheap.
    const int grid = dev->sm_count * 2;
    for (int d = 0; d < OCT_MAX_LEVEL; ++d) {
        k_tree_expand<<<grid, OT_THREADS, 0, s>>>(
            d, leaf_max, cap_nodes, keys.as<uint64_t>(), ctr.as<int>(), nd_start.as<int>(),
            nd_count.as<int>(), nd_depth.as<int>(), nd_parent.as<int>(), nd_rank.as<int>(),
            nd_int.as<int>(), in_node.as<int>(), in_nchild.as<int>());
        k_tree_mark<<<1, 32, 0, s>>>(d, ctr.as<int>());
    }
    GS_CUDA(cudaGetLastError());
    k_internal_keys<<<grid, OT_THREADS, 0, s>>>(ctr.as<int>(), in_node.as<int>(), nd_start.as<int>(),
                                                nd_depth.as<int>(), in_key.as<uint64_t>(),
                                                in_order.as<int>(), in_arrive.as<int>());
    GS_TRY(sorter.sort(in_key.as<uint64_t>(), in_order.as<int>(), ctr.as<int>() + CTR_SAFE_INTERNAL,
                       cap_nodes, internal_key_bits(),
                       reinterpret_cast<unsigned *>(ctr.as<int>() + CTR_STATUS), s));
    const int tiles = (cap_nodes + SCAN_TILE - 1) / SCAN_TILE;
    k_fc_tile_sums<<<tiles, OT_THREADS, 0, s>>>(ctr.as<int>(), in_order.as<int>(),
                                                in_nchild.as<int>(), scan_tiles.as<unsigned>());
    k_scan_small<<<1, 1024, 0, s>>>(scan_tiles.as<unsigned>(), tiles);
    k_fc_apply<<<tiles, OT_THREADS, 0, s>>>(ctr.as<int>(), in_order.as<int>(), in_nchild.as<int>(),
                                            scan_tiles.as<unsigned>(), in_fc.as<int>());
    k_tree_number<<<grid, OT_THREADS, 0, s>>>(
        ctr.as<int>(), compat ? 1 : 0, nd_start.as<int>(), nd_count.as<int>(), nd_depth.as<int>(),
        nd_parent.as<int>(), nd_rank.as<int>(), nd_int.as<int>(), in_nchild.as<int>(),
        in_fc.as<int>(), in_id.as<int>(), t_np.as<int>(), t_nc.as<int>(), t_fp.as<int>(),
        t_fc.as<int>(), t_depth.as<int>(), t_int.as<int>(), t_mass.as<double>(),
        t_com.as<double>());
    GS_CUDA(cudaGetLastError());
    if (links)
        k_tree_links<<<grid, OT_THREADS, 0, s>>>(ctr.as<int>(), nd_start.as<int>(),
                                                 nd_count.as<int>(), nd_parent.as<int>(),
                                                 nd_rank.as<int>(), nd_int.as<int>(),
                                                 in_node.as<int>(), in_fc.as<int>(),
                                                 t_parent.as<int>(), leaf_of.as<int>());
    MultipoleArgs A;
    A.xm = xm.as<double>();
    A.sidx = sidx.as<int>();
    A.in_node = in_node.as<int>();
    A.nd_parent = nd_parent.as<int>();
    A.in_id = in_id.as<int>();
    A.in_fc = in_fc.as<int>();
    A.in_nchild = in_nchild.as<int>();
    A.t_np = t_np.as<int>();
    A.t_nc = t_nc.as<int>();
    A.t_fp = t_fp.as<int>();
    A.t_int = t_int.as<int>();
    A.t_depth = t_depth.as<int>();
    A.frame = frame.as<double>();
    A.in_arrive = in_arrive.as<int>();
    A.in_sum = in_sum.as<double>();
    A.t_mass = t_mass.as<double>();
    A.t_com = t_com.as<double>();
    A.na = w_na.as<float4>();
    A.nb = w_nb.as<float4>();
    A.nq = quad ? w_nq.as<float4>() : nullptr;
    // particle records first: the leaves' quadrupoles are formed from them
    GS_CUDA(cudaMemsetAsync(mlist.p, 0, sizeof(int), s));
    k_walk_particles<<<pb, OT_THREADS, 0, s>>>(n, frame.as<double>(), d_x, d_m, sidx.as<int>(),
                                               w_pa.as<float4>(), w_pb.as<float4>(),
                                               xm.as<double>(), misplaced.as<unsigned char>(),
                                               mlist.as<int>());
    if (!compat)
        k_leaf_multipoles<<<grid, OT_THREADS, 0, s>>>(ctr.as<int>(), A, w_pa.as<float4>(),
                                                      w_pb.as<float4>());
    // four lanes per internal node: a larger grid, so that every node of a
    // tree of up to about 2^16 internal nodes starts at once
    k_multipole_up<<<dev->sm_count * 8, OT_THREADS, 0, s>>>(ctr.as<int>(), A);
    k_walk_nodes<<<grid, OT_THREADS, 0, s>>>(
        ctr.as<int>(), compat ? 1 : 0, frame.as<double>(), keys.as<uint64_t>(), sidx.as<int>(),
        t_np.as<int>(), t_nc.as<int>(), t_fp.as<int>(), t_fc.as<int>(), t_depth.as<int>(),
        t_mass.as<double>(), t_com.as<double>(), w_na.as<float4>(), w_nb.as<float4>(),
        w_nc.as<int4>(), w_nkey.as<uint64_t>());
    GS_CUDA(cudaGetLastError());
    return ok();
}

ErrorStatus OctreeDevice::read_counts(cudaStream_t s, int *nodes, unsigned *status)
{
    int h[3];
    GS_CUDA(cudaMemcpyAsync(h, ctr.p, sizeof(h), cudaMemcpyDeviceToHost, s));
    GS_CUDA(cudaStreamSynchronize(s));
    if (nodes) *nodes = h[CTR_NODES];
    if (status) *status = (unsigned)h[CTR_STATUS];
    return ok();
}

ErrorStatus OctreeDevice::clear_status(cudaStream_t s)
{
    GS_CUDA(cudaMemsetAsync(ctr.as<int>() + CTR_STATUS, 0, sizeof(int), s));
    GS_CUDA(cudaStreamSynchronize(s));
    return ok();
}

// Self-check of div_by_width against the division it replaces: per sample,
// a width w (a random significand, every tenth one all ones, an exponent in
// [-100, 100]) and a dividend x (a random 64-bit pattern for even k: every
// class of double; for odd k one whose quotient lies next to a midpoint of
// two doubles), the frame built as k_bbox_final builds it.
__device__ __forceinline__ unsigned long long wmix(unsigned long long z)
{
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__global__ void k_width_div_selftest(long long n, unsigned long long seed, unsigned long long *bad)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    unsigned long long local = 0;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += stride) {
        const unsigned long long h = wmix(seed ^ wmix((unsigned long long)k));
        unsigned long long sig = wmix(h + 7) >> 12;
        if (h % 10 == 0) sig = (1ull << 52) - 1ull;
        const int ew = (int)(wmix(h + 3) % 201) - 100;
        const double w = scalbn(__longlong_as_double((long long)(0x3ff0000000000000ull | sig)), ew);
        double frame[8];
        frame[3] = w;
        frame[5] = __ddiv_rn(1.0, w);
        frame[6] = __ddiv_rn(__fma_rn(-frame[5], w, 1.0), w);
        frame[7] = 1.0;
        double x;
        if (k & 1) {
            const unsigned long long m = (wmix(h + 11) >> 11) | (1ull << 52);
            const int e = (int)(wmix(h + 13) % 241) - 120;
            const double q0 = scalbn((double)m, e - 52);
            x = __fma_rn(q0, w, __dmul_rn(scalbn(1.0, e - 53), w));
        } else {
            x = __longlong_as_double((long long)wmix(h + 17));
        }
        const double a = div_by_width(x, frame), b = __ddiv_rn(x, w);
        const bool ok = (isnan(a) && isnan(b)) || __double_as_longlong(a) == __double_as_longlong(b);
        local += ok ? 0 : 1;
    }
    if (local) atomicAdd(bad, local);
}

}  // namespace gs

extern "C" int gsgpu_width_division_selftest(long long n, unsigned long long seed,
                                             long long *mismatches)
{
    if (!mismatches || n < 0) return GRAV_POINTER_ERROR;
    gs::DBuf bad;
    ErrorStatus st = bad.reserve(sizeof(unsigned long long));
    if (st.return_code != GRAV_SUCCESS) {
        free_traceback(&st);
        return GRAV_MEMORY_ERROR;
    }
    cudaError_t e = cudaMemset(bad.p, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) {
        gs::k_width_div_selftest<<<1216, 256>>>(n, seed, bad.as<unsigned long long>());
        e = cudaGetLastError();
    }
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, bad.p, sizeof(h), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        std::fprintf(stderr, "gsgpu_width_division_selftest: %s\n", cudaGetErrorString(e));
        return GRAV_FAILURE;
    }
    *mismatches = (long long)h;
    return GRAV_SUCCESS;
}

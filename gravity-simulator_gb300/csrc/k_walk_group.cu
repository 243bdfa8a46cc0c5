// k_walk_group.cu -- group Barnes-Hut walk with interaction lists
// (GRAV_GPU_BARNES_HUT_GROUP).
//
// The per-particle walk of k_walk.cu reproduces the reference's decisions
// (src/acceleration_barnes_hut.c:78-248) one child at a time, which costs
// about 200 instructions per accepted cell.  This walk trades identical
// decisions for throughput:
//   * groups come from the tree: in a cell with more than 32 particles,
//     each run of consecutive children of at most 32 particles is cut into
//     pieces of 32 sorted particles (a leaf with more is cut the same way),
//     so a group lies in one cell and its box stays compact where the
//     Morton curve jumps, and groups fill the lanes;
//     the one group that does not fit its cell (the particles whose Morton
//     coordinate wraps at the box maximum) is walked particle by particle;
//   * a persistent warp takes groups from a work queue and walks the tree
//     once per group, 32 nodes per step (one per lane), with the group
//     opening criterion
//         accept node  <=>  the node holds none of the group's particles
//                           (sorted ranges disjoint) and
//                           side^2 < theta^2 * dist(com, group box)^2,
//     which implies the per-particle criterion side^2 < theta^2 |com - x|^2
//     of the reference for every particle of the group, so the accepted
//     cells are at least as well separated as the reference's;
//   * accepted cells (centre of mass, mass, traceless quadrupole) and the
//     particles of opened leaves go to interaction lists in shared memory
//     (structure of arrays); when a list is full every lane evaluates it
//     against its own particle, two entries at a time through paired FP32
//     operations on float2 (broadcast shared-memory loads, dense FMA work),
//     and adds the partial sum to a Kahan-compensated accumulator;
//   * coordinates are FP32 offsets from the group's first particle, formed
//     from the frame-centred double-float (hi, lo) copies of the tree, so
//     near-field differences keep FP32 relative accuracy.
// Every wait is on __syncwarp only; a traversal stack that would overflow
// sets ST_STACK_OVERFLOW and ends the warp's walk (no spin, no trap).
#include "gs_octree.h"
#include "gs_ptx.cuh"

#include <atomic>

namespace gs {

constexpr int GW_WARPS = 4;        // groups per CTA
constexpr int GW_STACK = 1024;     // traversal stack entries per warp
constexpr int GW_CELLS = 128;      // cell list capacity per warp
constexpr int GW_PARTS = 128;      // particle list capacity per warp
// Stack entries kept free for a depth-first descent: popping one node and
// pushing its (at most 8) children grows the stack by 7 per level, over at
// most OCT_MAX_LEVEL + 1 levels.  Batches shrink so that the stack never
// passes GW_STACK - GW_RESERVE before such a descent starts, hence never
// overflows.
constexpr int GW_RESERVE = 8 * (OCT_MAX_LEVEL + 1);

constexpr int GW_GROUP = 32;       // particles per group at most

// Whether the particles of [first, first + count) lie within the side of a
// depth-`depth` cell, from their positions.
__device__ bool group_extent_fits(int first, int count, int depth, const float4 *__restrict__ pa,
                                  const float4 *__restrict__ pb, double box_length)
{
    const float4 oh = pa[first], ol = pb[first];
    float lo[3] = {0.f, 0.f, 0.f}, hi[3] = {0.f, 0.f, 0.f};
#pragma unroll 8
    for (int p = first + 1; p < first + count; ++p) {
        const float4 ph = pa[p], pl = pb[p];
        const float r[3] = {(ph.x - oh.x) + (pl.x - ol.x), (ph.y - oh.y) + (pl.y - ol.y),
                            (ph.z - oh.z) + (pl.z - ol.z)};
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], r[k]);
            hi[k] = fmaxf(hi[k], r[k]);
        }
    }
    const float ext = fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
    const double side = box_length / (double)(2 << min(depth, OCT_MAX_LEVEL + 1));
    return (double)ext * (double)ext <= 1.0001 * side * side;
}

// Group list: one thread per node.  A cell with more than GW_GROUP
// particles cuts each run of consecutive children of at most GW_GROUP
// particles into pieces of GW_GROUP (a leaf with more is cut the same way);
// the root is one group when it is small enough.  Entry: (first sorted particle,
// count | depth << 8) with depth that of the cell the group lies in.
// A group whose particles do not fit within the side of its cell (the
// particles whose Morton coordinate wraps at the box maximum sit in a cell
// on the far side) goes to the queue as single particles, so that no warp
// walks a box-wide group and its walks spread over the warps.
//
// A group's particles lie in one key cell, so it fits the cell's side unless
// it holds a particle whose key cell is not where it is (misplaced).  With at
// most kMisplacedCap of those (their sorted positions in mlist), only a group
// that holds one has its extent measured; the others fit without reading
// their particles.  With more, every group is measured.
__device__ void put_group(int2 *groups, int *gctr, int first, int count, int depth,
                          const float4 *__restrict__ pa, const float4 *__restrict__ pb,
                          double box_length, const int *__restrict__ mlist, int nmis)
{
    bool measure = nmis > kMisplacedCap;
    for (int k = 0; k < nmis && !measure; ++k) {
        const int q = mlist[1 + k];
        measure = q >= first && q < first + count;
    }
    const bool fits = !measure || group_extent_fits(first, count, depth, pa, pb, box_length);
    if (fits) {
        groups[atomicAdd(&gctr[0], 1)] = make_int2(first, count | (depth << 8));
    } else {
        const int at = atomicAdd(&gctr[0], count);
        for (int q = 0; q < count; ++q) groups[at + q] = make_int2(first + q, 1 | (depth << 8));
    }
}


__global__ void k_group_list(const int *__restrict__ ctr, const int4 *__restrict__ nc,
                             const int *__restrict__ depth, const float4 *__restrict__ pa,
                             const float4 *__restrict__ pb, const double *__restrict__ frame,
                             const int *__restrict__ mlist, int2 *__restrict__ groups,
                             int *__restrict__ gctr)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= tree_nodes(ctr)) return;   // no groups from an overflowed build
    const double bl = frame[4];
    const int nmis = mlist[0];
    const int4 ci = nc[c];   // (first child, children, first particle, particles)
    if (ci.w <= 0) return;
    const int d = depth[c];
    if (c == 0 && ci.w <= GW_GROUP) {
        put_group(groups, gctr, ci.z, ci.w, d, pa, pb, bl, mlist, nmis);
        return;
    }
    if (ci.w <= GW_GROUP) return;   // its own parent groups it
    if (ci.y <= 0) {                // oversized leaf (depth limit): runs of GW_GROUP
        for (int b = 0; b < ci.w; b += GW_GROUP)
            put_group(groups, gctr, ci.z + b, min(GW_GROUP, ci.w - b), d, pa, pb, bl, mlist, nmis);
        return;
    }
    // Runs of consecutive children of at most GW_GROUP particles each are
    // contiguous in sorted order and lie in this cell: each run is cut into
    // pieces of GW_GROUP particles (the last one shorter), so that groups
    // fill the warp's lanes (children of 20, 20 and 20 particles make groups
    // of 32 and 28, not three of 20).
    int first = 0, count = 0;
    for (int k = 0; k <= ci.y; ++k) {
        const int4 ch = k < ci.y ? nc[ci.x + k] : make_int4(0, 0, 0, GW_GROUP + 1);
        if (ch.w > GW_GROUP) {   // a child walked as its own cell, or the end
            for (int b = 0; b < count; b += GW_GROUP)
                put_group(groups, gctr, first + b, min(GW_GROUP, count - b), d, pa, pb, bl, mlist,
                          nmis);
            count = 0;
            continue;
        }
        if (ch.w <= 0) continue;
        if (count == 0) first = ch.z;
        count += ch.w;
    }
}

struct GroupWalkArgs {
    const float4 *na;       // (com_hi, mass)
    const float4 *nb;       // (com_lo, (cell side)^2)
    const float4 *nq;       // 2 per node: (xx, xy, xz, yy), (yz, zz, -, -)
    const int4 *nc;         // (first child, children, first particle, particles)
    const int *depth;
    const float4 *pa;       // sorted particles (x_hi, m)
    const float4 *pb;       // (x_lo, 0)
    const int *sidx;
    const double *frame;
    int n;
    float eps2;
    float theta2;
    double G;
    double *a;
    unsigned long long *counters;
    unsigned *status;
    const int *gate;        // when set, the launch runs only if *gate != 0
    const int2 *groups;     // (first sorted particle, count)
    int *gctr;              // [0] groups, [1] work-queue head
};

// Lists hold their entries in pairs: pair k is entries (2k, 2k+1), and each
// float4 carries two fields of both entries side by side, so that one
// 16-byte shared load gives two fields of the pair in the register pairs the
// paired FP32 operations read (half the loads of one float2 per field).
struct GroupShared {
    int stack[GW_STACK];
    float4 cA[GW_CELLS / 2];   // (x, x', y, y')        cell centre of mass
    float4 cB[GW_CELLS / 2];   // (z, z', m, m')        and mass
    float4 qA[GW_CELLS / 2];   // (xx, xx', xy, xy')    negated quadrupole
    float4 qB[GW_CELLS / 2];   // (xz, xz', yy, yy')
    float4 qC[GW_CELLS / 2];   // (yz, yz', zz, zz')
    float4 pA[GW_PARTS / 2];   // (x, x', y, y')        leaf particles
    float4 pB[GW_PARTS / 2];   // (z, z', m, m')
};
static_assert(GW_CELLS % 2 == 0 && GW_PARTS % 2 == 0, "lists hold whole pairs");

// Field f (0: the float4's first two lanes, 1: its last two) of entry j.
__device__ __forceinline__ void put(float4 *arr, int j, int f, float v)
{
    reinterpret_cast<float *>(arr)[(j >> 1) * 4 + 2 * f + (j & 1)] = v;
}

__device__ __forceinline__ float get(const float4 *arr, int j, int f)
{
    return reinterpret_cast<const float *>(arr)[(j >> 1) * 4 + 2 * f + (j & 1)];
}

__device__ __forceinline__ float2 lo2(const float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(const float4 v) { return make_float2(v.z, v.w); }

__device__ __forceinline__ float2 splat(float v) { return make_float2(v, v); }

// One cell term (monopole + optional quadrupole) for a lane's particle.
// The lists hold the negated quadrupole P = -Q; with d = com - x:
//     a = d [m / r^3 - 2.5 (d.P.d) / r^7] + P d / r^5
// (the monopole plus G [-Q d / r^5 + 2.5 (d.Q.d) d / r^7], G applied last).
template <bool QUAD>
__device__ __forceinline__ void cell_term1(const GroupShared &g, int j, float rx, float ry, float rz,
                                           float eps2, float &ax, float &ay, float &az)
{
    const float dx = get(g.cA, j, 0) - rx, dy = get(g.cA, j, 1) - ry, dz = get(g.cB, j, 0) - rz;
    const float ns = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float ri = rsqrt_approx(ns + eps2);
    const float ri2 = ri * ri;
    const float ri3 = ri2 * ri;
    float sc = get(g.cB, j, 1) * ri3;
    if (QUAD) {
        const float xx = get(g.qA, j, 0), xy = get(g.qA, j, 1), xz = get(g.qB, j, 0);
        const float yy = get(g.qB, j, 1), yz = get(g.qC, j, 0), zz = get(g.qC, j, 1);
        const float px = fmaf(xx, dx, fmaf(xy, dy, xz * dz));
        const float py = fmaf(xy, dx, fmaf(yy, dy, yz * dz));
        const float pz = fmaf(xz, dx, fmaf(yz, dy, zz * dz));
        const float dpd = fmaf(dx, px, fmaf(dy, py, dz * pz));
        const float ri5 = ri3 * ri2;
        sc = fmaf(-2.5f, dpd * (ri5 * ri2), sc);
        ax = fmaf(dx, sc, fmaf(px, ri5, ax));
        ay = fmaf(dy, sc, fmaf(py, ri5, ay));
        az = fmaf(dz, sc, fmaf(pz, ri5, az));
    } else {
        ax = fmaf(dx, sc, ax);
        ay = fmaf(dy, sc, ay);
        az = fmaf(dz, sc, az);
    }
}

template <bool QUAD>
__device__ __forceinline__ void flush_cells(const GroupShared &g, int count, float rx, float ry,
                                            float rz, float eps2, float &sx, float &cx, float &sy,
                                            float &cy, float &sz, float &cz)
{
    const float2 nrx = splat(-rx), nry = splat(-ry), nrz = splat(-rz), e2 = splat(eps2);
    float2 ax = splat(0.f), ay = splat(0.f), az = splat(0.f);
    int j = 0;
#pragma unroll 4
    for (; j + 1 < count; j += 2) {
        const float4 ca = g.cA[j >> 1], cb = g.cB[j >> 1];
        const float2 dx = __fadd2_rn(lo2(ca), nrx);
        const float2 dy = __fadd2_rn(hi2(ca), nry);
        const float2 dz = __fadd2_rn(lo2(cb), nrz);
        const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
        const float2 ri = make_float2(rsqrt_approx(r2.x), rsqrt_approx(r2.y));
        const float2 ri2 = __fmul2_rn(ri, ri);
        const float2 ri3 = __fmul2_rn(ri2, ri);
        float2 sc = __fmul2_rn(hi2(cb), ri3);
        if (QUAD) {
            // negated quadrupole P (see cell_term1)
            const float4 qa = g.qA[j >> 1], qb = g.qB[j >> 1], qc = g.qC[j >> 1];
            const float2 xx = lo2(qa), xy = hi2(qa), xz = lo2(qb);
            const float2 yy = hi2(qb), yz = lo2(qc), zz = hi2(qc);
            const float2 px = __ffma2_rn(xx, dx, __ffma2_rn(xy, dy, __fmul2_rn(xz, dz)));
            const float2 py = __ffma2_rn(xy, dx, __ffma2_rn(yy, dy, __fmul2_rn(yz, dz)));
            const float2 pz = __ffma2_rn(xz, dx, __ffma2_rn(yz, dy, __fmul2_rn(zz, dz)));
            const float2 dpd = __ffma2_rn(dx, px, __ffma2_rn(dy, py, __fmul2_rn(dz, pz)));
            const float2 ri5 = __fmul2_rn(ri3, ri2);
            sc = __ffma2_rn(splat(-2.5f), __fmul2_rn(dpd, __fmul2_rn(ri5, ri2)), sc);
            ax = __ffma2_rn(dx, sc, __ffma2_rn(px, ri5, ax));
            ay = __ffma2_rn(dy, sc, __ffma2_rn(py, ri5, ay));
            az = __ffma2_rn(dz, sc, __ffma2_rn(pz, ri5, az));
        } else {
            ax = __ffma2_rn(dx, sc, ax);
            ay = __ffma2_rn(dy, sc, ay);
            az = __ffma2_rn(dz, sc, az);
        }
    }
    float tx = ax.x + ax.y, ty = ay.x + ay.y, tz = az.x + az.y;
    if (j < count) cell_term1<QUAD>(g, j, rx, ry, rz, eps2, tx, ty, tz);
    kahan_add(sx, cx, tx);
    kahan_add(sy, cy, ty);
    kahan_add(sz, cz, tz);
}

// Leaf particles.  With softening every r^2 >= eps^2 > 0 and the particle's
// own term is 0 by its zero offset; without it the own term (r^2 = 0) is
// skipped explicitly.
template <bool SOFT>
__device__ __forceinline__ void flush_parts(const GroupShared &g, int count, float rx, float ry,
                                            float rz, float eps2, float &sx, float &cx, float &sy,
                                            float &cy, float &sz, float &cz)
{
    const float2 nrx = splat(-rx), nry = splat(-ry), nrz = splat(-rz), e2 = splat(eps2);
    float2 ax = splat(0.f), ay = splat(0.f), az = splat(0.f);
    int j = 0;
#pragma unroll 4
    for (; j + 1 < count; j += 2) {
        const float4 pa = g.pA[j >> 1], pb = g.pB[j >> 1];
        const float2 dx = __fadd2_rn(lo2(pa), nrx);
        const float2 dy = __fadd2_rn(hi2(pa), nry);
        const float2 dz = __fadd2_rn(lo2(pb), nrz);
        const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
        float2 ri = make_float2(rsqrt_approx(r2.x), rsqrt_approx(r2.y));
        if (!SOFT) {   // own term without softening: r2 = 0 contributes nothing
            ri.x = r2.x > 0.0f ? ri.x : 0.0f;
            ri.y = r2.y > 0.0f ? ri.y : 0.0f;
        }
        const float2 sc = __fmul2_rn(hi2(pb), __fmul2_rn(__fmul2_rn(ri, ri), ri));
        ax = __ffma2_rn(dx, sc, ax);
        ay = __ffma2_rn(dy, sc, ay);
        az = __ffma2_rn(dz, sc, az);
    }
    float tx = ax.x + ax.y, ty = ay.x + ay.y, tz = az.x + az.y;
    if (j < count) {
        const float dx = get(g.pA, j, 0) - rx, dy = get(g.pA, j, 1) - ry, dz = get(g.pB, j, 0) - rz;
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
        const float ri = (SOFT || r2 > 0.0f) ? rsqrt_approx(r2) : 0.0f;
        const float sc = get(g.pB, j, 1) * ri * ri * ri;
        tx = fmaf(dx, sc, tx);
        ty = fmaf(dy, sc, ty);
        tz = fmaf(dz, sc, tz);
    }
    kahan_add(sx, cx, tx);
    kahan_add(sy, cy, ty);
    kahan_add(sz, cz, tz);
}

// Walk of one group: sorted particles [g0, gend) on lanes 0..gend-g0-1.
template <bool QUAD, bool SOFT>
__device__ void walk_group(const GroupWalkArgs &A, GroupShared &g, const float *s_w2, int lane,
                           int g0, int gend)
{
    const int s = g0 + lane;
    const bool valid = s < gend;
    // origin: the group's first particle (double-float)
    const float4 oh = A.pa[g0], ol = A.pb[g0];
    float rx = 0.f, ry = 0.f, rz = 0.f;
    if (valid) {
        const float4 ph = A.pa[s], pl = A.pb[s];
        rx = (ph.x - oh.x) + (pl.x - ol.x);
        ry = (ph.y - oh.y) + (pl.y - ol.y);
        rz = (ph.z - oh.z) + (pl.z - ol.z);
    }
    float bx0 = valid ? rx : 3.0e38f, by0 = valid ? ry : 3.0e38f, bz0 = valid ? rz : 3.0e38f;
    float bx1 = valid ? rx : -3.0e38f, by1 = valid ? ry : -3.0e38f, bz1 = valid ? rz : -3.0e38f;
    for (int o = 16; o > 0; o >>= 1) {
        bx0 = fminf(bx0, __shfl_xor_sync(0xffffffffu, bx0, o));
        by0 = fminf(by0, __shfl_xor_sync(0xffffffffu, by0, o));
        bz0 = fminf(bz0, __shfl_xor_sync(0xffffffffu, bz0, o));
        bx1 = fmaxf(bx1, __shfl_xor_sync(0xffffffffu, bx1, o));
        by1 = fmaxf(by1, __shfl_xor_sync(0xffffffffu, by1, o));
        bz1 = fmaxf(bz1, __shfl_xor_sync(0xffffffffu, bz1, o));
    }
    const float th2 = A.theta2;
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    unsigned long long n_cell = 0, n_pp = 0;

    if (lane == 0) g.stack[0] = 0;   // root
    int top = 1, ncell = 0, npart = 0;
    __syncwarp();
    while (top > 0) {
        // pop k nodes, leaving room for up to 8 children of each
        int k = min(32, top);
        const int room = (GW_STACK - GW_RESERVE - top) / 7;
        if (room < k) k = max(1, room);
        const int node = lane < k ? g.stack[top - k + lane] : -1;
        top -= k;
        __syncwarp();
        int act = 0;   // 1 accept, 2 leaf, 3 open
        int4 ci = make_int4(0, 0, 0, 0);
        float4 crel = make_float4(0.f, 0.f, 0.f, 0.f);
        // quadrupole of the node, loaded with the node (used if accepted), so
        // that its latency overlaps the other loads instead of following the
        // decision
        float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = q0;
        if (node >= 0) {
            if (QUAD) {
                q0 = A.nq[2 * node];
                q1 = A.nq[2 * node + 1];
            }
            const float4 ca = A.na[node], cb = A.nb[node];
            ci = A.nc[node];
            crel = make_float4((ca.x - oh.x) + (cb.x - ol.x), (ca.y - oh.y) + (cb.y - ol.y),
                               (ca.z - oh.z) + (cb.z - ol.z), ca.w);
            const bool own = ci.z < gend && ci.z + ci.w > g0;
            const float ex = fmaxf(fmaxf(bx0 - crel.x, crel.x - bx1), 0.f);
            const float ey = fmaxf(fmaxf(by0 - crel.y, crel.y - by1), 0.f);
            const float ez = fmaxf(fmaxf(bz0 - crel.z, crel.z - bz1), 0.f);
            const float d2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
            const float w2 = cb.w;   // (cell side)^2 of the node's depth
            if (!own && w2 < th2 * d2 && ca.w > 0.f)
                act = 1;
            else if (ci.y <= 0)
                act = (ci.w > 0) ? 2 : 0;
            else
                act = 3;
            if (!own && ca.w <= 0.f && w2 < th2 * d2) act = 0;   // empty cell: nothing to add
        }
        // accepted cells
        const unsigned acc = __ballot_sync(0xffffffffu, act == 1);
        if (acc) {
            if (ncell + __popc(acc) > GW_CELLS) {
                __syncwarp();
                if (valid) flush_cells<QUAD>(g, ncell, rx, ry, rz, A.eps2, sx, cx, sy, cy, sz, cz);
                n_cell += valid ? ncell : 0;
                ncell = 0;
                __syncwarp();
            }
            if (act == 1) {
                const int at = ncell + __popc(acc & ((1u << lane) - 1u));
                put(g.cA, at, 0, crel.x);
                put(g.cA, at, 1, crel.y);
                put(g.cB, at, 0, crel.z);
                put(g.cB, at, 1, crel.w);
                if (QUAD) {   // negated, as the evaluation expects
                    put(g.qA, at, 0, -q0.x);
                    put(g.qA, at, 1, -q0.y);
                    put(g.qB, at, 0, -q0.z);
                    put(g.qB, at, 1, -q0.w);
                    put(g.qC, at, 0, -q1.x);
                    put(g.qC, at, 1, -q1.y);
                }
            }
            ncell += __popc(acc);
        }
        // particles of leaves that are not accepted
        const int cnt = (act == 2) ? ci.w : 0;
        int incl = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        if (total > 0) {
            if (total <= GW_PARTS) {
                if (npart + total > GW_PARTS) {
                    __syncwarp();
                    if (valid) flush_parts<SOFT>(g, npart, rx, ry, rz, A.eps2, sx, cx, sy, cy, sz, cz);
                    n_pp += valid ? npart : 0;
                    npart = 0;
                    __syncwarp();
                }
                // The warp copies the step's leaf particles together, one slot
                // per lane per round: slot t belongs to the last lane whose
                // exclusive prefix is <= t (found by a binary search over the
                // lanes), so every lane issues its loads at once.
                const int excl = incl - cnt;
                for (int base = 0; base < total; base += 32) {
                    const int t = base + lane;
                    int lo = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        const int e = __shfl_sync(0xffffffffu, excl, lo + step);
                        if (e <= t) lo += step;
                    }
                    const int first = __shfl_sync(0xffffffffu, ci.z, lo);
                    const int off = t - __shfl_sync(0xffffffffu, excl, lo);
                    if (t < total) {
                        const int p = first + off;
                        const float4 qa = A.pa[p], qb = A.pb[p];
                        const int at = npart + t;
                        put(g.pA, at, 0, (qa.x - oh.x) + (qb.x - ol.x));
                        put(g.pA, at, 1, (qa.y - oh.y) + (qb.y - ol.y));
                        put(g.pB, at, 0, (qa.z - oh.z) + (qb.z - ol.z));
                        put(g.pB, at, 1, qa.w);
                    }
                }
                npart += total;
                __syncwarp();
            } else {
                // large leaves: one lane's leaf at a time, 32 particles per round
                unsigned leaves = __ballot_sync(0xffffffffu, cnt > 0);
                while (leaves) {
                    const int src = __ffs(leaves) - 1;
                    leaves &= leaves - 1;
                    const int first = __shfl_sync(0xffffffffu, ci.z, src);
                    const int num = __shfl_sync(0xffffffffu, cnt, src);
                    for (int b = 0; b < num; b += 32) {
                        const int m32 = min(32, num - b);
                        if (npart + m32 > GW_PARTS) {
                            __syncwarp();
                            if (valid)
                                flush_parts<SOFT>(g, npart, rx, ry, rz, A.eps2, sx, cx, sy, cy, sz, cz);
                            n_pp += valid ? npart : 0;
                            npart = 0;
                            __syncwarp();
                        }
                        if (lane < m32) {
                            const int p = first + b + lane;
                            const float4 qa = A.pa[p], qb = A.pb[p];
                            const int at = npart + lane;
                            put(g.pA, at, 0, (qa.x - oh.x) + (qb.x - ol.x));
                            put(g.pA, at, 1, (qa.y - oh.y) + (qb.y - ol.y));
                            put(g.pB, at, 0, (qa.z - oh.z) + (qb.z - ol.z));
                            put(g.pB, at, 1, qa.w);
                        }
                        npart += m32;
                        __syncwarp();
                    }
                }
            }
        }
        // children of opened nodes
        const int ch = (act == 3) ? ci.y : 0;
        int cin = ch;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, cin, o);
            if (lane >= o) cin += t;
        }
        const int pushes = __shfl_sync(0xffffffffu, cin, 31);
        if (top + pushes > GW_STACK) {
            if (lane == 0) atomicOr(A.status, ST_STACK_OVERFLOW);
            break;
        }
        for (int q = 0; q < ch; ++q) g.stack[top + cin - ch + q] = ci.x + q;
        top += pushes;
        __syncwarp();
    }
    __syncwarp();
    if (valid && ncell > 0) flush_cells<QUAD>(g, ncell, rx, ry, rz, A.eps2, sx, cx, sy, cy, sz, cz);
    if (valid && npart > 0) flush_parts<SOFT>(g, npart, rx, ry, rz, A.eps2, sx, cx, sy, cy, sz, cz);
    if (valid) {
        n_cell += ncell;
        n_pp += npart - 1;   // every particle meets itself once in its own leaf
        const int id = A.sidx[s];
        A.a[3 * id + 0] = A.G * ((double)sx - (double)cx);
        A.a[3 * id + 1] = A.G * ((double)sy - (double)cy);
        A.a[3 * id + 2] = A.G * ((double)sz - (double)cz);
    }
    for (int o = 16; o > 0; o >>= 1) {
        n_cell += __shfl_down_sync(0xffffffffu, n_cell, o);
        n_pp += __shfl_down_sync(0xffffffffu, n_pp, o);
    }
    if (lane == 0) {
        atomicAdd(&A.counters[0], n_cell);
        atomicAdd(&A.counters[1], n_pp);
    }
    __syncwarp();   // every lane is done with the lists before the next group
}

// Whether the particles of a group lie within the side of the cell holding
// it.  A particle at the bounding-box maximum has its Morton coordinate
// wrapped to 0 (as in the reference) and sits in a cell on the far side; the
// group holding it spans the whole box and is walked one particle at a time.
__device__ bool group_fits(const GroupWalkArgs &A, const float *s_w2, int lane, int g0, int cnt,
                           int depth)
{
    const bool valid = lane < cnt;
    float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    if (valid) {
        const float4 oh = A.pa[g0], ol = A.pb[g0];
        const float4 ph = A.pa[g0 + lane], pl = A.pb[g0 + lane];
        const float r[3] = {(ph.x - oh.x) + (pl.x - ol.x), (ph.y - oh.y) + (pl.y - ol.y),
                            (ph.z - oh.z) + (pl.z - ol.z)};
        for (int k = 0; k < 3; ++k) lo[k] = hi[k] = r[k];
    }
    float ext = 0.f;
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
        ext = fmaxf(ext, hi[k] - lo[k]);
    }
    return ext * ext <= 1.0001f * s_w2[min(depth, OCT_MAX_LEVEL + 1)];
}

template <bool QUAD, bool SOFT>
// Five CTAs per SM (shared memory allows five; the register cap costs a few
// spilled bytes but keeps the fifth CTA resident).
__global__ void __launch_bounds__(32 * GW_WARPS, 5)
k_bh_group(GroupWalkArgs A)
{
    extern __shared__ __align__(16) unsigned char gw_smem[];
    __shared__ float s_w2[OCT_MAX_LEVEL + 2];   // (cell side at depth d)^2
    if (A.gate && *A.gate == 0) return;          // block-uniform
    GroupShared &g = reinterpret_cast<GroupShared *>(gw_smem)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    if (threadIdx.x <= OCT_MAX_LEVEL + 1) {
        // side of a depth-d cell: box_length / (2 << d)
        const double w = A.frame[4] / (double)(2 << threadIdx.x);
        s_w2[threadIdx.x] = (float)(w * w);
    }
    __syncthreads();
    const int ngroups = A.gctr[0];
    for (;;) {
        int gi = 0;
        if (lane == 0) gi = atomicAdd(&A.gctr[1], 1);
        gi = __shfl_sync(0xffffffffu, gi, 0);
        if (gi >= ngroups) break;   // warp-uniform
        const int2 grp = A.groups[gi];
        const int cnt = grp.y & 255, depth = grp.y >> 8;
        if (group_fits(A, s_w2, lane, grp.x, cnt, depth)) {
            walk_group<QUAD, SOFT>(A, g, s_w2, lane, grp.x, grp.x + cnt);
        } else {
            for (int q = 0; q < cnt; ++q)
                walk_group<QUAD, SOFT>(A, g, s_w2, lane, grp.x + q, grp.x + q + 1);
        }
    }
}

ErrorStatus launch_bh_group_walk(const OctreeDevice &t, double theta, double eps, double G,
                                 double *d_a, unsigned long long *counters, cudaStream_t s,
                                 const int *gate, bool reuse_groups)
{
    static_assert(sizeof(GroupShared) % 16 == 0, "group shared block alignment");
    const size_t smem = sizeof(GroupShared) * GW_WARPS;
    // The attribute belongs to the current device: set on every call (cheap,
    // host-side only, allowed during stream capture).
    const bool soft = eps > 0.0 && (float)(eps * eps) > 0.0f;
    auto kernel = t.quad ? (soft ? k_bh_group<true, true> : k_bh_group<true, false>)
                         : (soft ? k_bh_group<false, true> : k_bh_group<false, false>);
    GS_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    GroupWalkArgs w;
    w.na = t.w_na.as<float4>();
    w.nb = t.w_nb.as<float4>();
    w.nq = t.quad ? t.w_nq.as<float4>() : nullptr;
    w.nc = t.w_nc.as<int4>();
    w.depth = t.t_depth.as<int>();
    w.pa = t.w_pa.as<float4>();
    w.pb = t.w_pb.as<float4>();
    w.sidx = t.sidx.as<int>();
    w.frame = t.frame.as<double>();
    w.n = t.n;
    w.eps2 = (float)(eps * eps);
    w.theta2 = (float)(theta * theta);
    w.G = G;
    w.a = d_a;
    w.counters = counters;
    w.status = reinterpret_cast<unsigned *>(t.ctr.as<int>() + CTR_STATUS);
    w.gate = gate;
    w.groups = t.g_list.as<int2>();
    w.gctr = t.g_ctr.as<int>();
    if (reuse_groups) {
        // the list and its count stay; only the work-queue head restarts
        GS_CUDA(cudaMemsetAsync(w.gctr + 1, 0, sizeof(int), s));
    } else {
        GS_CUDA(cudaMemsetAsync(t.g_ctr.p, 0, 2 * sizeof(int), s));
        k_group_list<<<(t.cap_nodes + 255) / 256, 256, 0, s>>>(
            t.ctr.as<int>(), t.w_nc.as<int4>(), t.t_depth.as<int>(), t.w_pa.as<float4>(),
            t.w_pb.as<float4>(), t.frame.as<double>(), t.mlist.as<int>(), t.g_list.as<int2>(),
            w.gctr);
    }
    // persistent: every SM filled once (computed once per device)
    const DeviceInfo *dev = nullptr;
    GS_TRY(device_info(&dev));
    static std::atomic<int> grid_cache[kMaxDevices];
    int grid = grid_cache[dev->id].load(std::memory_order_acquire);
    if (grid == 0) {
        int per_sm = 0;
        GS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bh_group<true, true>,
                                                              32 * GW_WARPS, smem));
        grid = dev->sm_count * (per_sm > 0 ? per_sm : 1);
        grid_cache[dev->id].store(grid, std::memory_order_release);
    }
    kernel<<<grid, 32 * GW_WARPS, smem, s>>>(w);
    GS_CUDA(cudaGetLastError());
    return ok();
}

}  // namespace gs

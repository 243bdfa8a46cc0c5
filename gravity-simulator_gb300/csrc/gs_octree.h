// gs_octree.h -- device linear octree shared by the tree build (k_octree.cu)
// and the Barnes-Hut walk (k_walk.cu).
#pragma once

#include "gs_internal.h"
#include "gs_radix.h"

namespace gs {

constexpr int OCT_MAX_LEVEL = 21;   // MORTON_MAX_LEVEL (src/linear_octree.h:14)

// Device counters / small state of one build (ints unless noted).
enum OctCtr {
    CTR_NODES = 0,      // nodes created (root included)
    CTR_INTERNAL = 1,   // internal (expanded) nodes
    CTR_STATUS = 2,     // StatusBits
    CTR_N = 3,          // particle count (for device-count kernels)
    CTR_SAFE_INTERNAL = 4,   // internal nodes for the kernels after the expansion:
                             // CTR_INTERNAL, or 0 once the node capacity overflowed
    CTR_LVL = 8,        // CTR_LVL + d: first internal index of depth d (d = 0..22)
    CTR_SIZE = 40
};

#ifdef __CUDACC__
// A build whose node capacity overflowed leaves its counters past the
// capacity and its arrays partly written.  Every kernel after the expansion
// reads its node counts through these, so it does no work on such a build and
// stays inside the buffers; the status word keeps ST_TREE_OVERFLOW until the
// host reports it.
__device__ __forceinline__ bool tree_failed(const int *ctr)
{
    return (ctr[CTR_STATUS] & ST_TREE_OVERFLOW) != 0;
}
__device__ __forceinline__ int tree_nodes(const int *ctr)
{
    return tree_failed(ctr) ? 0 : ctr[CTR_NODES];
}
#endif

constexpr int kMisplacedCap = 64;

struct OctreeDevice {
    int n = 0;
    int cap_nodes = 0;   // node capacity
    int leaf_max = 1;
    bool compat = true;
    bool quad = false;   // traceless quadrupoles about the centre of mass
    DBuf w_nq;           // float4[2*cap]: (xx, xy, xz, yy), (yz, zz, 0, 0), FP32
    bool links = false;  // parent ids and particle -> leaf map
    ForceTimer *tm_morton = nullptr, *tm_sort = nullptr;   // build timing (optional)
    DBuf t_parent;       // int[cap] (-1 for the root)
    DBuf leaf_of;        // int[n]: leaf id of sorted particle p

    DBuf ctr;                 // int[CTR_SIZE]
    DBuf frame;               // double[8]: cx, cy, cz, width, box_length
    DBuf bbox_part;           // double[blocks * 6]
    DBuf keys, sidx;          // uint64[n] sorted Morton keys, int[n] particle ids
    // construction lists (unordered)
    DBuf nd_start, nd_count, nd_depth, nd_parent, nd_rank, nd_int;   // int[cap]
    DBuf in_node, in_nchild, in_fc, in_id;                           // int[cap]
    DBuf in_key;                                                     // uint64[cap]
    DBuf in_order;                                                   // int[cap]
    DBuf scan_tiles;                                                 // unsigned[...]
    // final node arrays in the reference's numbering
    DBuf t_np, t_nc, t_fp, t_fc, t_depth, t_int;                     // int[cap]
    DBuf t_mass;                                                     // double[cap]
    DBuf t_com;                                                      // double[3*cap]
    DBuf in_sum;                                                     // double[4*cap]
    DBuf in_arrive;   // int[cap]: children whose multipoles are done (bottom-up pass)
    // walk arrays (frame-centred double-float positions)
    DBuf w_na, w_nb;          // float4[cap]: (com_hi, mass), (com_lo, (cell side)^2)
    DBuf w_nc;                // int4[cap]: (first_child, num_children, first_particle, count)
    DBuf w_nkey;              // uint64[cap]: key used by the cell-membership test
    DBuf w_pa, w_pb;          // float4[n] in sorted order: (x_hi, m), (x_lo, 0)
    DBuf xm;                  // double[4n] in sorted order: x, y, z, m (the multipole sums' input)
    DBuf g_list;              // int2[n]: particle groups of the group walk (first, count)
    DBuf g_ctr;               // int[4]: group count, work-queue head
    // Particles whose Morton coordinate left [0, 2^21) and was masked (the
    // coordinate at the box maximum wraps to 0; a particle outside a given
    // box): their key cell is not where they are.  misplaced: uint8[n] by
    // particle id; mlist: int[1 + kMisplacedCap], the count and the sorted
    // positions of the first kMisplacedCap of them.
    DBuf misplaced, mlist;
    RadixSorter sorter;

    ErrorStatus setup(int n, int leaf_max, bool compat, bool quad = false);
    // Builds the tree from device x [3n] and m [n].  box_center/box_width
    // (host values) replace the bounding box when box_width > 0.
    ErrorStatus build(const double *d_x, const double *d_m, cudaStream_t s,
                      const double *box_center = nullptr, double box_width = -1.0);
    int launches_per_build() const;
    // Bits of the internal-node sort key (first particle << 5 | depth).
    int internal_key_bits() const
    {
        int b = 1;
        while (b < 31 && (1 << b) <= n) ++b;
        return b + 5;
    }
    // Host copies: number of nodes, status word.
    ErrorStatus read_counts(cudaStream_t s, int *nodes, unsigned *status);
    // Clears the status word once the host has reported it.
    ErrorStatus clear_status(cudaStream_t s);
};

// Barnes-Hut walk of a built tree (k_walk.cu).  counters (2 x u64) receive
// cell and particle terms (added); gate (device int, may be null) makes the
// launch return at once when *gate == 0.
ErrorStatus launch_bh_walk(const OctreeDevice &t, const double *d_x, double theta, double eps,
                           double G, double *d_a, const int *gate,
                           unsigned long long *counters, cudaStream_t s);

// Group walk with interaction lists (k_walk_group.cu): same counters and
// gate as launch_bh_walk; needs a tree with true leaf multipoles (not compat).
// The groups depend on the tree alone: a second walk of the same tree (another
// angle) passes reuse_groups and keeps the first walk's list.
ErrorStatus launch_bh_group_walk(const OctreeDevice &t, double theta, double eps, double G,
                                 double *d_a, unsigned long long *counters, cudaStream_t s,
                                 const int *gate = nullptr, bool reuse_groups = false);

}  // namespace gs

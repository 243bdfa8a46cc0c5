// k_walk.cu -- Barnes-Hut tree walk and the Barnes-Hut engine.
//
// Replaces helper_compute_acceleration (src/acceleration_barnes_hut.c:78-248)
// and acceleration_barnes_hut (:33-76).
//
// Warp-cooperative walk.  A warp owns 32 consecutive particles in Morton
// order and walks the union of their traversals: a warp-uniform stack holds,
// per depth, the node being scanned, the next child to scan and the mask of
// lanes still inside that subtree.  At each child every lane in the mask
// makes the reference's own decision for its particle --
//   cell-membership test on Morton prefixes (compat: the reference's
//   sorted-keys-by-particle-id read, :120/:145), then the opening test
//   (w_level)^2 < theta^2 |R|^2 (:157-162) -> monopole (:164-174),
//   else leaf -> particle terms skipping itself (:181-214), else descend --
// and the warp descends into the child when any lane needs it.  Each
// particle therefore sees exactly the nodes, in exactly the order, of the
// reference's depth-first walk; lanes not in a subtree's mask idle there.
//
// Precision: positions and centres of mass are double-float pairs (hi, lo)
// relative to the bounding-box centre, so R = (c_hi - x_hi) + (c_lo - x_lo)
// keeps FP32 relative accuracy for close pairs; pair terms are FP32 with
// rsqrt; each child's contribution is added to a Kahan-compensated FP32
// accumulator.  The opening test is made in FP32 unless |w^2 - theta^2|R|^2|
// is within 1e-5 of w^2, in which case it is recomputed in FP64 exactly as
// the reference does, so every decision equals the reference's.
#include "gs_octree.h"
#include "gs_ptx.cuh"

#include <cstdlib>
#include <cstring>

namespace gs {

constexpr int WK_THREADS = 128;
constexpr int WK_WARPS = WK_THREADS / 32;
constexpr int WK_STACK = OCT_MAX_LEVEL + 2;

struct WalkArgs {
    const float4 *na;
    const float4 *nb;
    const float4 *nq;       // quadrupoles (2 float4 per node) or null
    const int4 *nc;
    const uint64_t *nkey;
    const double *ncom;     // FP64 centre of mass [3*nodes] (exact opening test)
    const float4 *pa;
    const float4 *pb;
    const int *sidx;
    const uint64_t *skeys;  // sorted keys
    const double *x;        // FP64 positions by particle id
    const double *frame;    // cx, cy, cz, width, box_length
    int n;
    int compat;
    float eps2;
    double theta2;
    double G;
    double *a;
    unsigned long long *counters;   // [0] accepted cells, [1] leaf pair terms
    unsigned *status;
    const int *gate;                // when set, the launch runs only if *gate != 0
};

__device__ __forceinline__ void add3(float &sx, float &cx, float &sy, float &cy, float &sz, float &cz,
                                     float px, float py, float pz)
{
    kahan_add(sx, cx, px);
    kahan_add(sy, cy, py);
    kahan_add(sz, cz, pz);
}

template <bool QUAD>
__global__ void __launch_bounds__(WK_THREADS)
k_bh_walk(WalkArgs A)
{
    __shared__ int s_node[WK_WARPS][WK_STACK];
    __shared__ int s_next[WK_WARPS][WK_STACK];
    __shared__ unsigned s_mask[WK_WARPS][WK_STACK];
    __shared__ float s_w2[WK_STACK];     // (cell width at depth)^2, FP32
    __shared__ double s_w[WK_STACK];     // cell width at depth, FP64 (reference formula)

    if (A.gate && *A.gate == 0) return;   // block-uniform
    if (*A.status & ST_TREE_OVERFLOW) return;   // the build overflowed: no tree to walk
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x < WK_STACK) {
        const int lv = threadIdx.x;
        // box_length / (2 << level)  (src/acceleration_barnes_hut.c:157)
        const double w = lv >= 1 && lv <= OCT_MAX_LEVEL ? __ddiv_rn(A.frame[4], (double)(2 << lv)) : 0.0;
        s_w[lv] = w;
        s_w2[lv] = __double2float_rn(__dmul_rn(w, w));
    }
    __syncthreads();

    const int s = blockIdx.x * WK_THREADS + threadIdx.x;
    const bool valid = s < A.n;
    const int id = valid ? A.sidx[s] : -1;
    uint64_t key_i = 0;
    float xh = 0.f, yh = 0.f, zh = 0.f, xl = 0.f, yl = 0.f, zl = 0.f;
    double x0 = 0.0, x1 = 0.0, x2 = 0.0;
    if (valid) {
        key_i = A.compat ? A.skeys[id] : A.skeys[s];
        const float4 ph = A.pa[s];
        const float4 pl = A.pb[s];
        xh = ph.x; yh = ph.y; zh = ph.z;
        xl = pl.x; yl = pl.y; zl = pl.z;
        x0 = A.x[3 * id + 0];
        x1 = A.x[3 * id + 1];
        x2 = A.x[3 * id + 2];
    }
    const float th2f = (float)A.theta2;
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    unsigned long long n_cell = 0, n_pp = 0;

    const unsigned valid_mask = __ballot_sync(0xffffffffu, valid);
    if (valid_mask == 0) return;
    if (lane == 0) {
        s_node[warp][0] = 0;
        s_next[warp][0] = 0;
        s_mask[warp][0] = valid_mask;
    }
    __syncwarp();
    int top = 0;
    int level = 1;   // depth of the children being scanned
    for (;;) {
        const int node = s_node[warp][top];
        const int nxt = s_next[warp][top];
        const int4 pinfo = A.nc[node];
        if (nxt >= pinfo.y) {
            if (top == 0) break;
            --top;
            --level;
            continue;
        }
        __syncwarp();
        if (lane == 0) s_next[warp][top] = nxt + 1;
        const unsigned mask = s_mask[warp][top];
        __syncwarp();
        const int c = pinfo.x + nxt;
        const bool act = (mask >> lane) & 1u;
        const float4 ca = A.na[c];
        const float4 cb = A.nb[c];
        const int4 ci = A.nc[c];
        const uint64_t ck = A.nkey[c];
        int dec = 0;   // 1 accepted, 2 leaf, 3 open
        if (act) {
            const int sh = 3 * (OCT_MAX_LEVEL - level);
            const bool inside = (key_i >> sh) == (ck >> sh);
            if (!inside) {
                const float dx = (ca.x - xh) + (cb.x - xl);
                const float dy = (ca.y - yh) + (cb.y - yl);
                const float dz = (ca.z - zh) + (cb.z - zl);
                const float ns = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                const float w2 = s_w2[level];
                const float t = th2f * ns;
                bool accept;
                if (fabsf(w2 - t) <= 1e-5f * w2) {
                    // exact FP64 test, reference operation order
                    const double r0 = __dsub_rn(x0, A.ncom[3 * c + 0]);
                    const double r1 = __dsub_rn(x1, A.ncom[3 * c + 1]);
                    const double r2 = __dsub_rn(x2, A.ncom[3 * c + 2]);
                    const double nsd = __dadd_rn(__dadd_rn(__dmul_rn(r0, r0), __dmul_rn(r1, r1)),
                                                 __dmul_rn(r2, r2));
                    const double wd = s_w[level];
                    accept = __dmul_rn(wd, wd) < __dmul_rn(A.theta2, nsd);
                } else {
                    accept = w2 < t;
                }
                if (accept) {
                    const float r2 = ns + A.eps2;
                    const float ri = rsqrt_approx(r2);
                    const float ri2 = ri * ri;
                    const float ri3 = ri2 * ri;
                    const float sc = ca.w * ri3;
                    float px = dx * sc, py = dy * sc, pz = dz * sc;
                    if (QUAD) {
                        // d = com - x = -R:  G [-Q d / r^5 + 2.5 (d.Q.d) d / r^7]
                        const float4 q0 = A.nq[2 * c];
                        const float4 q1 = A.nq[2 * c + 1];
                        const float qx = q0.x * dx + q0.y * dy + q0.z * dz;
                        const float qy = q0.y * dx + q0.w * dy + q1.x * dz;
                        const float qz = q0.z * dx + q1.x * dy + q1.y * dz;
                        const float dqd = dx * qx + dy * qy + dz * qz;
                        const float ri5 = ri3 * ri2;
                        const float f = 2.5f * dqd * ri5 * ri2;
                        px += f * dx - qx * ri5;
                        py += f * dy - qy * ri5;
                        pz += f * dz - qz * ri5;
                    }
                    add3(sx, cx, sy, cy, sz, cz, px, py, pz);
                    ++n_cell;
                    dec = 1;
                }
            }
            if (dec == 0) dec = (ci.y <= 0) ? 2 : 3;
        }
        const unsigned leaf_mask = __ballot_sync(0xffffffffu, dec == 2);
        const unsigned open_mask = __ballot_sync(0xffffffffu, dec == 3);
        if (leaf_mask) {
            float px = 0.f, py = 0.f, pz = 0.f;
            for (int k = 0; k < ci.w; ++k) {
                const int p = ci.z + k;
                const float4 qa = A.pa[p];
                const float4 qb = A.pb[p];
                const int pid = A.sidx[p];
                if (dec == 2 && pid != id) {
                    const float dx = (qa.x - xh) + (qb.x - xl);
                    const float dy = (qa.y - yh) + (qb.y - yl);
                    const float dz = (qa.z - zh) + (qb.z - zl);
                    const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, A.eps2)));
                    const float ri = rsqrt_approx(r2);
                    const float sc = qa.w * ri * ri * ri;
                    px = fmaf(dx, sc, px);
                    py = fmaf(dy, sc, py);
                    pz = fmaf(dz, sc, pz);
                    ++n_pp;
                }
            }
            if (dec == 2) add3(sx, cx, sy, cy, sz, cz, px, py, pz);
        }
        if (open_mask) {
            if (top + 1 >= WK_STACK) {
                if (lane == 0) atomicOr(A.status, ST_STACK_OVERFLOW);
                break;
            }
            ++top;
            ++level;
            __syncwarp();
            if (lane == 0) {
                s_node[warp][top] = c;
                s_next[warp][top] = 0;
                s_mask[warp][top] = open_mask;
            }
            __syncwarp();
        }
    }
    if (valid) {
        A.a[3 * id + 0] = A.G * ((double)sx - (double)cx);
        A.a[3 * id + 1] = A.G * ((double)sy - (double)cy);
        A.a[3 * id + 2] = A.G * ((double)sz - (double)cz);
    }
    // interaction counts (warp sums, one atomic per warp)
    for (int o = 16; o > 0; o >>= 1) {
        n_cell += __shfl_down_sync(0xffffffffu, n_cell, o);
        n_pp += __shfl_down_sync(0xffffffffu, n_pp, o);
    }
    if (lane == 0) {
        atomicAdd(&A.counters[0], n_cell);
        atomicAdd(&A.counters[1], n_pp);
    }
}

// ------------------------------------------------------------------------
namespace {

class BarnesHutEngine final : public Engine {
  public:
    BarnesHutEngine(bool compat, bool quad, bool group)
        : compat_(compat), quad_(quad && !compat), group_(group && !compat)
    {
    }

    ErrorStatus setup(int n, double G, const AccelerationParam &p) override
    {
        n_ = n;
        G_ = G;
        eps_ = p.softening_length;
        theta_ = p.opening_angle;
        GS_TRY(tree_.setup(n, p.max_num_particles_per_leaf, compat_, quad_));
        GS_TRY(counters_.reserve(4 * sizeof(unsigned long long)));
        GS_CUDA(cudaMemset(counters_.p, 0, 4 * sizeof(unsigned long long)));
        return ok();
    }

    ErrorStatus compute(const double *d_x, const double *d_m, double *d_a, cudaStream_t s,
                        ForceTimer *timer) override
    {
        GS_TRY(tree_.build(d_x, d_m, s));
        WalkArgs w;
        w.na = tree_.w_na.as<float4>();
        w.nb = tree_.w_nb.as<float4>();
        w.nq = quad_ ? tree_.w_nq.as<float4>() : nullptr;
        w.nc = tree_.w_nc.as<int4>();
        w.nkey = tree_.w_nkey.as<uint64_t>();
        w.ncom = tree_.t_com.as<double>();
        w.pa = tree_.w_pa.as<float4>();
        w.pb = tree_.w_pb.as<float4>();
        w.sidx = tree_.sidx.as<int>();
        w.skeys = tree_.keys.as<uint64_t>();
        w.x = d_x;
        w.frame = tree_.frame.as<double>();
        w.n = n_;
        w.compat = compat_ ? 1 : 0;
        w.eps2 = (float)(eps_ * eps_);
        w.theta2 = theta_ * theta_;
        w.G = G_;
        w.a = d_a;
        w.counters = counters_.as<unsigned long long>();
        w.status = reinterpret_cast<unsigned *>(tree_.ctr.as<int>() + CTR_STATUS);
        w.gate = nullptr;
        GS_CUDA(cudaMemsetAsync(counters_.p, 0, 2 * sizeof(unsigned long long), s));
        if (group_) {
            if (timer) GS_TRY(timer->begin(s));
            GS_TRY(launch_bh_group_walk(tree_, theta_, eps_, G_, d_a, w.counters, s));
            if (timer) GS_TRY(timer->end(s));
            return ok();
        }
        if (timer) GS_TRY(timer->begin(s));
        const int grid = (n_ + WK_THREADS - 1) / WK_THREADS;
        if (quad_)
            k_bh_walk<true><<<grid, WK_THREADS, 0, s>>>(w);
        else
            k_bh_walk<false><<<grid, WK_THREADS, 0, s>>>(w);
        GS_CUDA(cudaGetLastError());
        if (timer) GS_TRY(timer->end(s));
        return ok();
    }

    // the group walk is two launches (group list, walk)
    int kernels_per_eval() const override { return tree_.launches_per_build() + (group_ ? 2 : 1); }

    ErrorStatus check_status(cudaStream_t s) override
    {
        int nodes = 0;
        unsigned st = 0;
        GS_TRY(tree_.read_counts(s, &nodes, &st));
        if (st) GS_TRY(tree_.clear_status(s));
        if (st & ST_TREE_OVERFLOW)
            return GS_RAISE(GRAV_MEMORY_ERROR, "octree node capacity (%d) exceeded", tree_.cap_nodes);
        if (st & ST_STACK_OVERFLOW)
            return GS_RAISE(GRAV_FAILURE, "tree walk deeper than the octree depth limit");
        if (st & ST_WAIT_TIMEOUT)
            return GS_RAISE(GRAV_FAILURE, "octree key sort: a look-back wait ran out");
        return ok();
    }

    void set_build_timers(ForceTimer *morton, ForceTimer *sort) override
    {
        tree_.tm_morton = morton;
        tree_.tm_sort = sort;
    }

    ErrorStatus interaction_counts(cudaStream_t s, long long out[2]) override
    {
        unsigned long long h[2] = {0, 0};
        GS_CUDA(cudaMemcpyAsync(h, counters_.p, sizeof(h), cudaMemcpyDeviceToHost, s));
        GS_CUDA(cudaStreamSynchronize(s));
        out[0] = (long long)h[0];
        out[1] = (long long)h[1];
        return ok();
    }

  private:
    bool compat_, quad_, group_;
    int n_ = 0;
    double G_ = 1.0, eps_ = 0.0, theta_ = 1.0;
    OctreeDevice tree_;
    DBuf counters_;
};

}  // namespace

std::unique_ptr<Engine> make_barnes_hut_engine(bool compat, bool quad, bool group)
{
    return std::unique_ptr<Engine>(new BarnesHutEngine(compat, quad, group));
}

// Walk of a built (non-compat) tree, for engines that walk one tree several
// times (the learned method's cheap walk and its gated fallback).
ErrorStatus launch_bh_walk(const OctreeDevice &t, const double *d_x, double theta, double eps,
                           double G, double *d_a, const int *gate,
                           unsigned long long *counters, cudaStream_t s)
{
    WalkArgs w;
    w.na = t.w_na.as<float4>();
    w.nb = t.w_nb.as<float4>();
    w.nq = t.quad ? t.w_nq.as<float4>() : nullptr;
    w.nc = t.w_nc.as<int4>();
    w.nkey = t.w_nkey.as<uint64_t>();
    w.ncom = t.t_com.as<double>();
    w.pa = t.w_pa.as<float4>();
    w.pb = t.w_pb.as<float4>();
    w.sidx = t.sidx.as<int>();
    w.skeys = t.keys.as<uint64_t>();
    w.x = d_x;
    w.frame = t.frame.as<double>();
    w.n = t.n;
    w.compat = t.compat ? 1 : 0;
    w.eps2 = (float)(eps * eps);
    w.theta2 = theta * theta;
    w.G = G;
    w.a = d_a;
    w.counters = counters;
    w.status = reinterpret_cast<unsigned *>(t.ctr.as<int>() + CTR_STATUS);
    w.gate = gate;
    const int grid = (t.n + WK_THREADS - 1) / WK_THREADS;
    if (t.quad)
        k_bh_walk<true><<<grid, WK_THREADS, 0, s>>>(w);
    else
        k_bh_walk<false><<<grid, WK_THREADS, 0, s>>>(w);
    GS_CUDA(cudaGetLastError());
    return ok();
}

ErrorStatus accel_host(double *a, const System *system, const AccelerationParam *param_in);

// construct_octree on the GPU, copied to host arrays the caller frees with
// free_linear_octree (src/linear_octree.c:825-976).
ErrorStatus octree_to_host(const AccelerationParam &p_in, const System *system,
                           const double *box_center, double box_width, LinearOctree *out)
{
    if (!out) return GS_RAISE(GRAV_POINTER_ERROR, "Octree pointer is NULL");
    if (!system) return GS_RAISE(GRAV_POINTER_ERROR, "System pointer is NULL");
    if (system->num_particles <= 0 || !system->x || !system->m)
        return GS_RAISE(GRAV_VALUE_ERROR, "System has no particles");
    const int n = system->num_particles;
    const bool compat = p_in.method == ACCELERATION_METHOD_BARNES_HUT ||
                        p_in.method == GRAV_GPU_BARNES_HUT_COMPAT;
    int leaf = p_in.max_num_particles_per_leaf;
    if (leaf == -1) leaf = 1;
    if (leaf < 1)
        return GS_RAISE(GRAV_VALUE_ERROR,
                        "Maximum number of particles per leaf must be positive. Got: %d", leaf);
    OctreeDevice t;
    GS_TRY(t.setup(n, leaf, compat));
    DBuf dx, dm;
    GS_TRY(dx.reserve((size_t)n * 3 * sizeof(double)));
    GS_TRY(dm.reserve((size_t)n * sizeof(double)));
    cudaStream_t s = nullptr;
    GS_CUDA(cudaMemcpy(dx.p, system->x, (size_t)n * 3 * sizeof(double), cudaMemcpyHostToDevice));
    GS_CUDA(cudaMemcpy(dm.p, system->m, (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
    GS_TRY(t.build(dx.as<double>(), dm.as<double>(), s, box_center, box_width));
    int nodes = 0;
    unsigned st = 0;
    GS_TRY(t.read_counts(s, &nodes, &st));
    if (st & ST_TREE_OVERFLOW)
        return GS_RAISE(GRAV_MEMORY_ERROR, "octree node capacity (%d) exceeded", t.cap_nodes);
    if (st & ST_WAIT_TIMEOUT)
        return GS_RAISE(GRAV_FAILURE, "octree key sort: a look-back wait ran out");
    LinearOctree o;
    std::memset(&o, 0, sizeof(o));
    o.num_internal_nodes = nodes;
    o.particle_morton_indices_deepest_level = (int64_t *)std::malloc((size_t)n * sizeof(int64_t));
    o.sorted_indices = (int *)std::malloc((size_t)n * sizeof(int));
    o.tree_num_particles = (int *)std::malloc((size_t)nodes * sizeof(int));
    o.tree_num_internal_children = (int *)std::malloc((size_t)nodes * sizeof(int));
    o.tree_first_particle_sorted_idx = (int *)std::malloc((size_t)nodes * sizeof(int));
    o.tree_first_internal_children_idx = (int *)std::malloc((size_t)nodes * sizeof(int));
    o.tree_mass = (double *)std::malloc((size_t)nodes * sizeof(double));
    o.tree_center_of_mass_x = (double *)std::malloc((size_t)nodes * sizeof(double));
    o.tree_center_of_mass_y = (double *)std::malloc((size_t)nodes * sizeof(double));
    o.tree_center_of_mass_z = (double *)std::malloc((size_t)nodes * sizeof(double));
    double *com = (double *)std::malloc((size_t)nodes * 3 * sizeof(double));
    double frame[8];
    if (!o.particle_morton_indices_deepest_level || !o.sorted_indices || !o.tree_num_particles ||
        !o.tree_num_internal_children || !o.tree_first_particle_sorted_idx ||
        !o.tree_first_internal_children_idx || !o.tree_mass || !o.tree_center_of_mass_x ||
        !o.tree_center_of_mass_y || !o.tree_center_of_mass_z || !com) {
        std::free(com);
        free_linear_octree(&o);
        return GS_RAISE(GRAV_MEMORY_ERROR, "Failed to allocate memory for the octree arrays");
    }
    cudaError_t e = cudaSuccess;
    e = e ? e : cudaMemcpy(o.particle_morton_indices_deepest_level, t.keys.p, (size_t)n * 8, cudaMemcpyDeviceToHost);
    e = e ? e : cudaMemcpy(o.sorted_indices, t.sidx.p, (size_t)n * 4, cudaMemcpyDeviceToHost);
    e = e ? e : cudaMemcpy(o.tree_num_particles, t.t_np.p, (size_t)nodes * 4, cudaMemcpyDeviceToHost);
    e = e ? e : cudaMemcpy(o.tree_num_internal_children, t.t_nc.p, (size_t)nodes * 4, cudaMemcpyDeviceToHost);
    e = e ? e : cudaMemcpy(o.tree_first_particle_sorted_idx, t.t_fp.p, (size_t)nodes * 4, cudaMemcpyDeviceToHost);
    e = e ? e : cudaMemcpy(o.tree_first_internal_children_idx, t.t_fc.p, (size_t)nodes * 4, cudaMemcpyDeviceToHost);
    e = e ? e : cudaMemcpy(o.tree_mass, t.t_mass.p, (size_t)nodes * 8, cudaMemcpyDeviceToHost);
    e = e ? e : cudaMemcpy(com, t.t_com.p, (size_t)nodes * 24, cudaMemcpyDeviceToHost);
    e = e ? e : cudaMemcpy(frame, t.frame.p, sizeof(frame), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        std::free(com);
        free_linear_octree(&o);
        GS_CUDA(e);
    }
    for (int i = 0; i < nodes; ++i) {
        o.tree_center_of_mass_x[i] = com[3 * i + 0];
        o.tree_center_of_mass_y[i] = com[3 * i + 1];
        o.tree_center_of_mass_z[i] = com[3 * i + 2];
    }
    std::free(com);
    o.box_width = frame[3];
    *out = o;
    return ok();
}

}  // namespace gs

using namespace gs;

extern "C" {

ErrorStatus acceleration_barnes_hut(double *a, const System *system,
                                    const AccelerationParam *acceleration_param)
{
    if (!acceleration_param)
        return GS_RAISE(GRAV_POINTER_ERROR, "Acceleration parameter pointer is NULL");
    AccelerationParam p = *acceleration_param;
    if (p.method == ACCELERATION_METHOD_BARNES_HUT || p.method == GRAV_GPU_BARNES_HUT_COMPAT)
        p.method = GRAV_GPU_BARNES_HUT_COMPAT;
    else
        p.method = GRAV_GPU_BARNES_HUT;
    return gs::accel_host(a, system, &p);
}

LinearOctree get_new_linear_octree(void)
{
    LinearOctree t;
    std::memset(&t, 0, sizeof(t));
    return t;
}

ErrorStatus construct_octree(LinearOctree *octree, const System *system,
                             const AccelerationParam *acceleration_param, const double *box_center,
                             double box_width)
{
    if (!acceleration_param)
        return GS_RAISE(GRAV_POINTER_ERROR, "Acceleration parameter pointer is NULL");
    return gs::octree_to_host(*acceleration_param, system, box_center, box_width, octree);
}

void free_linear_octree(LinearOctree *octree)
{
    if (!octree) return;
    std::free(octree->particle_morton_indices_deepest_level);
    std::free(octree->sorted_indices);
    std::free(octree->tree_num_particles);
    std::free(octree->tree_num_internal_children);
    std::free(octree->tree_first_particle_sorted_idx);
    std::free(octree->tree_first_internal_children_idx);
    std::free(octree->tree_mass);
    std::free(octree->tree_center_of_mass_x);
    std::free(octree->tree_center_of_mass_y);
    std::free(octree->tree_center_of_mass_z);
    std::memset(octree, 0, sizeof(*octree));
}

}  // extern "C"

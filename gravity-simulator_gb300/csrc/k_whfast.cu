// k_whfast.cu -- batched planetary ensembles: WHFast and leapfrog with the
// massless acceleration, many independent systems of uneven size per launch.
//
// Replaces whfast and its helpers (src/integrator_whfast.c:200-1279),
// system_sort_by_distance / remove_particles (src/system.c:444-577,
// :1210-1335), and for leapfrog acceleration_massless
// (src/acceleration.c:236-367) with the kicks / drifts of src/integrator.c.
//
// Layout: all systems concatenated; system s owns slots [off[s], off[s+1])
// of every per-particle array and its first cnt[s] slots are live (WHFast
// can remove particles).  Every kernel covers all systems in one launch
// (the sort: one launch per size class of systems):
//   k_wh_sort       one CTA per system: sort by distance from the primary
//                   (bitonic sort of (distance, index) in shared memory,
//                   ties by index), permute, eta (sequential prefix);
//   k_wh_seq_*      removals (compaction), eta, Jacobi <-> Cartesian
//                   recurrences, massive-body list: a warp per system for
//                   the scans and fills, a thread per system for the
//                   sequential steps of the recurrence;
//   k_wh_drift      one thread per particle: universal-variable Kepler
//                   solve (Newton, Stumpff series with argument quartering);
//   k_wh_accel      one thread per particle: interaction accelerations in
//                   Jacobi form (massless or pairwise variant);
//   k_wh_kick       v_jac += a dt.
// Every FP64 operation is an explicitly rounded intrinsic in the
// reference's expression order, so each system evolves exactly as the
// reference evolves it (where the reference is not FMA-contracted and does
// not read its uninitialised a[0] / aux, taken as zero here).
#include "gs_internal.h"
#include "gs_ptx.cuh"

#include <algorithm>
#include <cstdio>
#include <vector>

namespace gs {

// Ensemble integrator / acceleration variants.
enum { WH_MASSLESS = 0, WH_PAIRWISE = 1 };

// Largest system of an ensemble: the per-system sort holds 12 bytes per
// slot of the next power of two in shared memory (192 KiB at 16384).
constexpr int kEnsembleMaxSystem = 16384;

// Shared pair sums of the interaction acceleration (k_wh_pairs): used when a
// system has at most kPairMax massive bodies.
constexpr int kPairMax = 32;
constexpr int kPairSlots = kPairMax + 1;

struct EnsDev {
    int S;
    const int *off;      // [S+1]
    int *cnt;            // [S]
    const int *sys_of;   // [P]
    int *ids;
    double *x, *v, *m, *jx, *jv, *a, *eta;
    int *hv;             // massive-body list (indices within the system), per system at off[s]
    int *nh;             // [S]
    int *rm;             // [P] removal marks
    int *nrm;            // [S]
    double *pairs;       // [S][2 * kPairSlots][3] shared pair sums
    // Jacobi -> Cartesian pass (k_wh_seq_scan / _chain / _fill)
    int *seq_nmass;      // [S] massive particles (run path), -1: whole chain, -2: empty
    int *seq_runs;       // [S] massless runs recorded
    int *run_lo, *run_hi;   // [S][kSeqMassMax + 1] first / last slot of a run
    double *run_y;       // [S][kSeqMassMax + 1][6] offsets of a run's x and v
    // scratch for the permutation
    int *t_ids;
    double *t_x, *t_v, *t_m;
    unsigned *status;
    double G, eps;
    int variant;
    int remove_invalid;
};

__device__ __forceinline__ double dot3(const double *a, const double *b)
{
    return __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
}

__device__ __forceinline__ double norm3d(const double *a) { return __dsqrt_rn(dot3(a, a)); }

// ---- sort by distance ----------------------------------------------------
// Sort key of a distance: its bit pattern (distances are >= 0, so the
// patterns order like the values), NaN after +inf, padding after all.
// This keeps the comparison a total order whatever the input, so every
// live slot receives a live index.
__device__ __forceinline__ unsigned long long dist_key(double d)
{
    return isnan(d) ? 0x7ff8000000000000ull : (unsigned long long)__double_as_longlong(fabs(d));
}

// eta_i = m_0 + m_1 + ... + m_i, added one by one in slot order
// (src/integrator_whfast.c:1266-1279), from the masses in ms[0..n), by warp
// 0 of the block.  The warp walks the slots 32 at a time and performs only
// the adds that can change the running sum: adding +-0 to a sum that is
// neither zero nor NaN returns the sum itself, so massless slots repeat the
// sum of the last massive slot before them, and only the massive slots
// (and every slot while the sum is zero or NaN) are added, in order, with
// the reference's rounding.  The results are those of the one-by-one loop
// bit for bit; a system of test particles costs a few adds instead of n.
__device__ void sort_eta(const double *ms, double *eta, int n)
{
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    double e = ms[0];
    if (lane == 0) eta[0] = e;
    for (int c = 1; c < n; c += 32) {
        const int i = c + lane;
        const double mi = i < n ? ms[i] : 0.0;
        const unsigned valid = __ballot_sync(0xffffffffu, i < n);
        const unsigned nz = __ballot_sync(0xffffffffu, i < n && mi != 0.0);
        double mine = e;   // the sum after the last slot added at or before this lane
        int j = -1;
        for (;;) {
            const unsigned above = j < 0 ? 0xffffffffu : ~((2u << j) - 1u);   // lanes > j
            const bool every = e == 0.0 || isnan(e);
            const unsigned cand = (every ? valid : nz) & above;
            if (!cand) break;
            j = __ffs(cand) - 1;
            e = __dadd_rn(e, __shfl_sync(0xffffffffu, mi, j));
            if (lane >= j) mine = e;
        }
        if (i < n) eta[i] = mine;
    }
}

// Sorts slots of one system by |vec_i - vec_prim| and permutes vec, vel, m,
// ids; then eta.  Dynamic shared memory: pow2 * (8 + 4) bytes.
constexpr int SORT_OET_PASSES = 32;   // odd-even passes tried before the bitonic network

__global__ void k_wh_sort(EnsDev E, double *vec, double *vel, int pow2_max, int need_eta,
                          const int *__restrict__ systems)
{
    extern __shared__ __align__(16) unsigned char wh_smem[];
    const int s = systems[blockIdx.x];
    const int base = E.off[s];
    const int n = E.cnt[s];
    if (n <= 0) return;
    int P2 = 1;
    while (P2 < n) P2 <<= 1;
    if (P2 > pow2_max) {
        if (threadIdx.x == 0) atomicOr(E.status, ST_CAPACITY);
        return;
    }
    unsigned long long *key = reinterpret_cast<unsigned long long *>(wh_smem);
    int *idx = reinterpret_cast<int *>(wh_smem + (size_t)pow2_max * 8);
    __shared__ int prim_s;
    if (threadIdx.x == 0) {
        int prim = -1;
        if (E.ids[base] == 0) {
            prim = 0;
        } else {
            for (int i = 0; i < n; ++i)
                if (E.ids[base + i] == 0) {
                    prim = i;
                    break;
                }
        }
        prim_s = prim;
    }
    __syncthreads();
    const int prim = prim_s;
    if (prim < 0) {
        if (threadIdx.x == 0) atomicOr(E.status, ST_NO_PRIMARY);
        return;
    }
    const double p0 = vec[3 * (base + prim)], p1 = vec[3 * (base + prim) + 1],
                 p2 = vec[3 * (base + prim) + 2];
    for (int i = threadIdx.x; i < P2; i += blockDim.x) {
        if (i < n) {
            const double d[3] = {__dsub_rn(vec[3 * (base + i)], p0),
                                 __dsub_rn(vec[3 * (base + i) + 1], p1),
                                 __dsub_rn(vec[3 * (base + i) + 2], p2)};
            // first the squared distance, the radicand of the reference's key
            key[i] = (i == prim) ? 0ull : dist_key(dot3(d, d));
            idx[i] = i;
        } else {
            key[i] = ~0ull;   // padding sorts last
            idx[i] = 0x7fffffff;
        }
    }
    __syncthreads();
    // Already in order (the usual case from one step to the next): a stable
    // sort is the identity; eta is kept unless it was never formed.  The
    // square root is monotone, so squared distances in order imply distances
    // in order, and the check needs no square roots.  Otherwise the keys
    // become the distances themselves (rounded square roots can tie where
    // the squares did not) and are checked again.
    bool unsorted = false;
    for (int i = threadIdx.x; i + 1 < n; i += blockDim.x)
        unsorted = unsorted || key[i] > key[i + 1];
    if (__syncthreads_or(unsorted)) {
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            if (i != prim) key[i] = dist_key(__dsqrt_rn(__longlong_as_double((long long)key[i])));
        __syncthreads();
        unsorted = false;
        for (int i = threadIdx.x; i + 1 < n; i += blockDim.x)
            unsorted = unsorted || key[i] > key[i + 1];
    }
    if (!__syncthreads_or(unsorted)) {
        if (need_eta) {   // the keys are done with: their space holds the masses
            double *ms = reinterpret_cast<double *>(wh_smem);
            for (int i = threadIdx.x; i < n; i += blockDim.x) ms[i] = E.m[base + i];
            __syncthreads();
            sort_eta(ms, E.eta + base, n);
        }
        return;
    }
    // Nearly in order: odd-even transposition by (key, idx) until two
    // passes in a row swap nothing; the bitonic network finishes otherwise.
    int clean = 0;
    for (int pass = 0; pass < SORT_OET_PASSES && clean < 2; ++pass) {
        bool swapped = false;
        for (int i = (pass & 1) + 2 * threadIdx.x; i + 1 < n; i += 2 * blockDim.x) {
            const unsigned long long ka = key[i], kb = key[i + 1];
            const int ia = idx[i], ib = idx[i + 1];
            if (ka > kb || (ka == kb && ia > ib)) {
                key[i] = kb;
                key[i + 1] = ka;
                idx[i] = ib;
                idx[i + 1] = ia;
                swapped = true;
            }
        }
        clean = __syncthreads_or(swapped) ? 0 : clean + 1;
    }
    // bitonic sort ascending by (key, idx)
    for (int k = 2; clean < 2 && k <= P2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P2; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const bool up = (i & k) == 0;
                    const unsigned long long ki = key[i], kl = key[l];
                    const int ii = idx[i], il = idx[l];
                    const bool gt = (ki > kl) || (ki == kl && ii > il);
                    if (gt == up) {
                        key[i] = kl;
                        key[l] = ki;
                        idx[i] = il;
                        idx[l] = ii;
                    }
                }
            }
            __syncthreads();
        }
    }
    // permute through the scratch arrays
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int j = idx[i];
        if (j < 0 || j >= n) {   // unreachable with a total order; never read outside
            atomicOr(E.status, ST_NONFINITE);
            continue;
        }
        const int src = base + j, dst = base + i;
        E.t_ids[dst] = E.ids[src];
        E.t_m[dst] = E.m[src];
        for (int c = 0; c < 3; ++c) {
            E.t_x[3 * dst + c] = vec[3 * src + c];
            E.t_v[3 * dst + c] = vel[3 * src + c];
        }
    }
    __syncthreads();
    // the keys are done with: their space holds the permuted masses for eta
    double *ms = reinterpret_cast<double *>(wh_smem);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int d = base + i;
        E.ids[d] = E.t_ids[d];
        const double md = E.t_m[d];
        E.m[d] = md;
        ms[i] = md;
        for (int c = 0; c < 3; ++c) {
            vec[3 * d + c] = E.t_x[3 * d + c];
            vel[3 * d + c] = E.t_v[3 * d + c];
        }
    }
    __syncthreads();
    sort_eta(ms, E.eta + base, n);   // src/integrator_whfast.c:1266-1279
}

// ---- per-system sequential work ---------------------------------------------
// One warp per system.  The Jacobi recurrences are a chain through the
// interior centre of mass, so lane 0 runs the chain while the warp stages
// chunks of the system through shared memory with coalesced loads and
// stores; the massive-body list is built by ballots.
constexpr int SEQ_WARPS = 4;     // systems per CTA

// Massless runs of the Jacobi -> Cartesian chain.  For a particle with
// m_i = 0 (finite Jacobi coordinates, eta_i = eta_{i-1} = e, and a centre
// that is not -0, which subtracting +-0 would turn into +0) a chain step is
//     y = RN(xc / e),  x_i = jx_i + y,  xc <- RN(e y),
// and after a step or two xc is a fixed point of that map (checked bit for
// bit).  From there on every particle of the run adds the same y, so only
// the first steps of a run and the massive particles are sequential; the
// rest of the run is one add per coordinate, done by the whole warp.
constexpr int kSeqMassMax = 64;   // massive particles handled by the run path

struct SeqRuns {
    int mass_idx[kSeqMassMax];
    int lo[kSeqMassMax + 1], hi[kSeqMassMax + 1];
    double y[kSeqMassMax + 1][6];
    int nruns;
};

__device__ __forceinline__ bool neg_zero(double v)
{
    return __double_as_longlong(v) == (long long)0x8000000000000000ull;
}

// One exact chain step of src/integrator_whfast.c:744-760 for particle i;
// y[6] receives the offsets added to jx_i / jv_i.
__device__ __forceinline__ void jac_step(double xc[3], double vc[3], double mi, double ei,
                                         double ep, const double *jxi, const double *jvi,
                                         double *xi, double *vi, double y[6])
{
    for (int k = 0; k < 3; ++k) {
        xc[k] = __ddiv_rn(__dsub_rn(xc[k], __dmul_rn(mi, jxi[k])), ei);
        vc[k] = __ddiv_rn(__dsub_rn(vc[k], __dmul_rn(mi, jvi[k])), ei);
        y[k] = xc[k];
        y[3 + k] = vc[k];
        xi[k] = __dadd_rn(jxi[k], xc[k]);
        vi[k] = __dadd_rn(jvi[k], vc[k]);
        xc[k] = __dmul_rn(ep, xc[k]);
        vc[k] = __dmul_rn(ep, vc[k]);
    }
}

__device__ void wh_massive_list_warp(const EnsDev &E, int base, int n, int s, int lane)
{
    int k = 0;
    for (int c = 0; c < n; c += 32) {
        const int i = c + lane;
        const bool h = i < n && (E.variant == WH_PAIRWISE || E.m[base + i] != 0.0);
        const unsigned b = __ballot_sync(0xffffffffu, h);
        if (h) E.hv[base + k + __popc(b & ((1u << lane) - 1u))] = i;
        k += __popc(b);
    }
    if (lane == 0) E.nh[s] = k;
}

// Cartesian -> Jacobi, once per run; rebuilds the massive-body list.
__global__ void __launch_bounds__(32 * SEQ_WARPS) k_wh_seq_init(EnsDev E)
{
    __shared__ SeqRuns shared_all[SEQ_WARPS];
    const int lane = threadIdx.x & 31;
    const int s = blockIdx.x * SEQ_WARPS + (threadIdx.x >> 5);
    if (s >= E.S) return;   // warp-uniform
    SeqRuns &rs = shared_all[threadIdx.x >> 5];
    const int base = E.off[s];
    const int n = E.cnt[s];
    if (n <= 0) return;
    const double *m = E.m + base, *eta = E.eta + base;
    const double *x = E.x + 3 * base, *v = E.v + 3 * base;
    double *jx = E.jx + 3 * base, *jv = E.jv + 3 * base;
    {
        // src/integrator_whfast.c:682-724 (once per run).  For a massless
        // particle the interior centre of mass is left exactly as it is
        // (factor 1 + 0/eta = 1, added term +-0), so with finite
        // coordinates and a non-zero centre every particle of a massless run
        // subtracts the same y = xc / eta and the run is filled by the warp.
        bool finite0 = true;
        int nmass0 = 0;
        for (int c = 0; c < n; c += 32) {
            const int i = c + lane;
            bool f = true, h = false;
            if (i < n) {
                for (int k = 0; k < 3; ++k) f = f && isfinite(x[3 * i + k]) && isfinite(v[3 * i + k]);
                h = m[i] != 0.0;
            }
            finite0 = __all_sync(0xffffffffu, f) && finite0;
            const unsigned b = __ballot_sync(0xffffffffu, h);
            const int at = nmass0 + __popc(b & ((1u << lane) - 1u));
            if (h && at < kSeqMassMax) rs.mass_idx[at] = i;
            nmass0 += __popc(b);
        }
        if (finite0 && nmass0 <= kSeqMassMax) {
            __syncwarp();
            if (lane == 0) {
                double xc[3], vc[3];
                for (int k = 0; k < 3; ++k) {
                    xc[k] = __dmul_rn(m[0], x[k]);
                    vc[k] = __dmul_rn(m[0], v[k]);
                }
                int nr = 0, q = 0;
                int i = 1;
                while (i < n) {
                    while (q < nmass0 && rs.mass_idx[q] < i) ++q;
                    const int next_mass = q < nmass0 ? rs.mass_idx[q] : n;
                    // only a centre of -0 is changed by adding +-0 (to +0)
                    bool nz = true;
                    for (int k = 0; k < 3; ++k) nz = nz && !neg_zero(xc[k]) && !neg_zero(vc[k]);
                    if (next_mass > i && nz) {
                        // massless run [i, next_mass): one offset for all
                        const double ie = eta[i - 1];
                        rs.lo[nr] = i;
                        rs.hi[nr] = next_mass - 1;
                        for (int k = 0; k < 3; ++k) {
                            rs.y[nr][k] = __ddiv_rn(xc[k], ie);
                            rs.y[nr][3 + k] = __ddiv_rn(vc[k], ie);
                        }
                        ++nr;
                        i = next_mass;
                        continue;
                    }
                    const double ie = eta[i - 1];
                    for (int k = 0; k < 3; ++k) {
                        jx[3 * i + k] = __dsub_rn(x[3 * i + k], __ddiv_rn(xc[k], ie));
                        jv[3 * i + k] = __dsub_rn(v[3 * i + k], __ddiv_rn(vc[k], ie));
                        const double f = __dadd_rn(1.0, __ddiv_rn(m[i], ie));
                        xc[k] = __dadd_rn(__dmul_rn(xc[k], f), __dmul_rn(m[i], jx[3 * i + k]));
                        vc[k] = __dadd_rn(__dmul_rn(vc[k], f), __dmul_rn(m[i], jv[3 * i + k]));
                    }
                    ++i;
                }
                for (int k = 0; k < 3; ++k) {
                    jx[k] = __ddiv_rn(xc[k], eta[n - 1]);
                    jv[k] = __ddiv_rn(vc[k], eta[n - 1]);
                }
                rs.nruns = nr;
            }
            __syncwarp();
            const int nr = rs.nruns;
            for (int r = 0; r < nr; ++r) {
                const int lo = rs.lo[r], cnt = 3 * (rs.hi[r] - lo + 1);
                for (int t = lane; t < cnt; t += 32) {
                    const int k = t % 3;
                    jx[3 * lo + t] = __dsub_rn(x[3 * lo + t], rs.y[r][k]);
                    jv[3 * lo + t] = __dsub_rn(v[3 * lo + t], rs.y[r][3 + k]);
                }
            }
            __syncwarp();
            wh_massive_list_warp(E, base, n, s, lane);
            return;
        }
        __syncwarp();
        if (lane == 0) {
            double xc[3], vc[3];
            for (int k = 0; k < 3; ++k) {
                xc[k] = __dmul_rn(m[0], x[k]);
                vc[k] = __dmul_rn(m[0], v[k]);
            }
            for (int i = 1; i < n; ++i) {
                const double ie = eta[i - 1];
                for (int k = 0; k < 3; ++k) {
                    jx[3 * i + k] = __dsub_rn(x[3 * i + k], __ddiv_rn(xc[k], ie));
                    jv[3 * i + k] = __dsub_rn(v[3 * i + k], __ddiv_rn(vc[k], ie));
                    const double f = __dadd_rn(1.0, __ddiv_rn(m[i], ie));
                    xc[k] = __dadd_rn(__dmul_rn(xc[k], f), __dmul_rn(m[i], jx[3 * i + k]));
                    vc[k] = __dadd_rn(__dmul_rn(vc[k], f), __dmul_rn(m[i], jv[3 * i + k]));
                }
            }
            for (int k = 0; k < 3; ++k) {
                jx[k] = __ddiv_rn(xc[k], eta[n - 1]);
                jv[k] = __ddiv_rn(vc[k], eta[n - 1]);
            }
        }
        __syncwarp();
        wh_massive_list_warp(E, base, n, s, lane);
    }
}

// ---- Jacobi -> Cartesian, every step (src/integrator_whfast.c:726-772) --------
// The recurrence runs from the outermost particle inwards through the
// interior centre of mass xc, one particle after another.  Only a few of
// its steps are sequential work: a massless particle leaves the centre at a
// fixed point of xc <- RN(e RN(xc / e)) after a step or two, from where
// every particle of its massless run adds the same offset.  So the pass is
//   k_wh_seq_scan   one CTA per system: removals (compaction, eta), then
//                   finite Jacobi coordinates and the massive particles'
//                   slots in order (the massive-body list, and at most
//                   kSeqMassMax of them for the chain);
//   k_wh_seq_chain  one thread per system: the sequential steps (massive
//                   particles, and the first steps of each massless run until
//                   the fixed point), recording each run's offsets; the whole
//                   chain where the run path does not apply;
//   k_wh_seq_fill   one thread per slot: the runs (x = jx + offset).
// The chain is a lane's own work: FP64 instructions of a lane-0-only warp
// cost the FP64 pipe as much as a full warp's, so a warp of 32 systems'
// chains does 32 times the work of one system's chain in the same time.
constexpr int SCAN_THREADS = 128;

__global__ void __launch_bounds__(SCAN_THREADS) k_wh_seq_scan(EnsDev E)
{
    const int s = blockIdx.x;
    const int base = E.off[s];
    int n = E.cnt[s];
    if (n <= 0) {
        if (threadIdx.x == 0) E.seq_nmass[s] = -2;
        return;
    }
    double *m = E.m + base, *eta = E.eta + base;
    double *x = E.x + 3 * base, *v = E.v + 3 * base, *jx = E.jx + 3 * base, *jv = E.jv + 3 * base;
    const int nrm = E.nrm[s];
    __syncthreads();   // every thread has read nrm before thread 0 clears it
    if (nrm > 0) {
        // src/system.c:444-528 and :530-577: stable compaction of the
        // surviving slots (Cartesian x, v, m, ids, Jacobi x, v), then eta
        if (threadIdx.x == 0) {
            int w = 0;
            for (int i = 0; i < n; ++i) {
                if (E.rm[base + i]) {
                    E.rm[base + i] = 0;
                    continue;
                }
                if (w != i) {
                    E.ids[base + w] = E.ids[base + i];
                    m[w] = m[i];
                    for (int k = 0; k < 3; ++k) {
                        x[3 * w + k] = x[3 * i + k];
                        v[3 * w + k] = v[3 * i + k];
                        jx[3 * w + k] = jx[3 * i + k];
                        jv[3 * w + k] = jv[3 * i + k];
                    }
                }
                ++w;
            }
            E.cnt[s] = w;
            E.nrm[s] = 0;
            double e = m[0];
            eta[0] = e;
            for (int i = 1; i < w; ++i) {
                e = __dadd_rn(e, m[i]);
                eta[i] = e;
            }
        }
        __syncthreads();
        n = E.cnt[s];
    }
    // finite Jacobi coordinates (the run path needs them)
    bool f = true;
    for (int i = threadIdx.x; i < n; i += SCAN_THREADS)
        for (int k = 0; k < 3; ++k) f = f && isfinite(jx[3 * i + k]) && isfinite(jv[3 * i + k]);
    const bool finite = __syncthreads_and(f);
    // the slots with m != 0 in order: counts over contiguous ranges, an
    // exclusive scan over the block, then the writes
    const int per = (n + SCAN_THREADS - 1) / SCAN_THREADS;
    const int lo = min(n, (int)threadIdx.x * per), hi = min(n, lo + per);
    int c = 0;
    for (int i = lo; i < hi; ++i) c += m[i] != 0.0 ? 1 : 0;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = c;
    for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += t;
    }
    __shared__ int warp_tot[SCAN_THREADS / 32];
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    int at = incl - c, total = 0;
    for (int w = 0; w < SCAN_THREADS / 32; ++w) {
        if (w < wid) at += warp_tot[w];
        total += warp_tot[w];
    }
    int *mass_idx = E.t_ids + base;
    int *hv = E.hv + base;
    const bool massless = E.variant != WH_PAIRWISE;
    for (int i = lo; i < hi; ++i) {
        if (m[i] == 0.0) continue;
        if (at < kSeqMassMax) mass_idx[at] = i;
        if (massless) hv[at] = i;   // the massive-body list
        ++at;
    }
    if (!massless)
        for (int i = threadIdx.x; i < n; i += SCAN_THREADS) hv[i] = i;
    if (threadIdx.x == 0) {
        E.nh[s] = massless ? total : n;
        E.seq_nmass[s] = (finite && total <= kSeqMassMax) ? total : -1;
    }
}

__global__ void k_wh_seq_chain(EnsDev E)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= E.S) return;
    const int nmass = E.seq_nmass[s];
    if (nmass == -2) return;   // empty system
    const int base = E.off[s];
    const int n = E.cnt[s];
    const double *m = E.m + base, *eta = E.eta + base;
    double *x = E.x + 3 * base, *v = E.v + 3 * base;
    const double *jx = E.jx + 3 * base, *jv = E.jv + 3 * base;
    double xc[3], vc[3], y[6];
    for (int k = 0; k < 3; ++k) {
        xc[k] = __dmul_rn(eta[n - 1], jx[k]);
        vc[k] = __dmul_rn(eta[n - 1], jv[k]);
    }
    const size_t rb = (size_t)s * (kSeqMassMax + 1);
    int nr = 0;
    if (nmass >= 0) {
        const int *mass_idx = E.t_ids + base;
        int q = nmass - 1;   // highest massive particle not yet passed
        int i = n - 1;
        while (i >= 1) {
            while (q >= 0 && mass_idx[q] > i) --q;
            const int mtop = q >= 0 ? mass_idx[q] : -1;
            if (mtop == i) {
                jac_step(xc, vc, m[i], eta[i], eta[i - 1], jx + 3 * i, jv + 3 * i, x + 3 * i,
                         v + 3 * i, y);
                --i;
                continue;
            }
            const int lo = mtop + 1 > 1 ? mtop + 1 : 1;
            int j = i;
            bool fixed = false;
            while (j >= lo && !fixed) {
                const double ox[3] = {xc[0], xc[1], xc[2]}, ov[3] = {vc[0], vc[1], vc[2]};
                jac_step(xc, vc, m[j], eta[j], eta[j - 1], jx + 3 * j, jv + 3 * j, x + 3 * j,
                         v + 3 * j, y);
                fixed = true;
                for (int k = 0; k < 3; ++k)
                    fixed = fixed && __double_as_longlong(xc[k]) == __double_as_longlong(ox[k]) &&
                            __double_as_longlong(vc[k]) == __double_as_longlong(ov[k]) &&
                            isfinite(xc[k]) && isfinite(vc[k]) && !neg_zero(xc[k]) &&
                            !neg_zero(vc[k]);
                --j;
            }
            if (j >= lo) {
                E.run_lo[rb + nr] = lo;
                E.run_hi[rb + nr] = j;
                for (int k = 0; k < 6; ++k) E.run_y[(rb + nr) * 6 + k] = y[k];
                ++nr;
            }
            i = lo - 1;
        }
    } else {
        // the whole chain, particle by particle
        for (int i = n - 1; i >= 1; --i)
            jac_step(xc, vc, m[i], eta[i], eta[i - 1], jx + 3 * i, jv + 3 * i, x + 3 * i, v + 3 * i,
                     y);
    }
    E.seq_runs[s] = nr;
    for (int k = 0; k < 3; ++k) {
        x[k] = __ddiv_rn(xc[k], m[0]);
        v[k] = __ddiv_rn(vc[k], m[0]);
    }
}

// One thread per slot: a slot of a massless run takes the run's offsets.
__global__ void k_wh_seq_fill(EnsDev E, int P)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int s = E.sys_of[p];
    const int i = p - E.off[s];
    if (i >= E.cnt[s]) return;
    const int nr = E.seq_runs[s];
    const size_t rb = (size_t)s * (kSeqMassMax + 1);
    for (int r = 0; r < nr; ++r) {
        if (i < E.run_lo[rb + r] || i > E.run_hi[rb + r]) continue;
        const double *y = E.run_y + (rb + r) * 6;
        for (int k = 0; k < 3; ++k) {
            E.x[3 * (size_t)p + k] = __dadd_rn(E.jx[3 * (size_t)p + k], y[k]);
            E.v[3 * (size_t)p + k] = __dadd_rn(E.jv[3 * (size_t)p + k], y[3 + k]);
        }
        return;
    }
}

// ---- shared interaction pair sums ---------------------------------------------
// The pair term of the interaction acceleration (src/integrator_whfast.c
// :1125-1190 / :920-950) sums over interior massive bodies j and exterior
// massive bodies k of particle i; it depends on i only through which massive
// bodies are interior.  So it is formed once per system and partition, in
// the reference's (j, k) order, and every particle with that partition reads
// the same bits:
//   slot g (1 <= g <= nh)         a particle with g interior massive bodies
//                                  that is not itself massive;
//   slot kPairSlots + r (r >= 1)  the massive body of list rank r.

constexpr int PAIR_WARPS = 2;   // systems per CTA
constexpr int kPairTerms = kPairMax * (kPairMax - 1) / 2;

// One warp per system: every massive pair term G m_j m_k (x_k - x_j) /
// (|x_k - x_j|^3 + eps^3) once into shared memory (pair (p, q), p < q in
// list order, at q (q - 1) / 2 + p), then one lane per slot adds its terms
// in the reference's order.
__global__ void __launch_bounds__(32 * PAIR_WARPS) k_wh_pairs(EnsDev E)
{
    __shared__ double terms_all[PAIR_WARPS][kPairTerms][3];
    const int lane = threadIdx.x & 31;
    const int s = blockIdx.x * PAIR_WARPS + (threadIdx.x >> 5);
    if (s >= E.S) return;   // warp-uniform
    const int nh = E.nh[s];
    if (nh > kPairMax) return;
    double(*terms)[3] = terms_all[threadIdx.x >> 5];
    const int base = E.off[s];
    const double *x = E.x + 3 * (size_t)base;
    const double *m = E.m + base;
    const int *hv = E.hv + base;
    const double e3 = __dmul_rn(__dmul_rn(E.eps, E.eps), E.eps);
    const int npairs = nh * (nh - 1) / 2;
    for (int t = lane; t < npairs; t += 32) {
        int q = 1;
        while ((q + 1) * q / 2 <= t) ++q;
        const int p = t - q * (q - 1) / 2;
        const int j = hv[p], kk = hv[q];
        const double d[3] = {__dsub_rn(x[3 * kk], x[3 * j]), __dsub_rn(x[3 * kk + 1], x[3 * j + 1]),
                             __dsub_rn(x[3 * kk + 2], x[3 * j + 2])};
        const double dn = norm3d(d);
        const double dc = __dadd_rn(__dmul_rn(__dmul_rn(dn, dn), dn), e3);
        const double Gmm = __dmul_rn(__dmul_rn(E.G, m[j]), m[kk]);
        for (int k = 0; k < 3; ++k) terms[t][k] = __ddiv_rn(__dmul_rn(Gmm, d[k]), dc);
    }
    __syncwarp();
    for (int slot = lane; slot < 2 * kPairSlots; slot += 32) {
        int p_end, q_begin;
        if (slot < kPairSlots) {
            if (slot > nh) continue;
            p_end = slot;
            q_begin = slot;
        } else {
            const int r = slot - kPairSlots;
            if (r >= nh) continue;
            p_end = r;
            q_begin = r + 1;
        }
        double aux[3] = {0.0, 0.0, 0.0};
        for (int p = 0; p < p_end; ++p)
            for (int q = q_begin; q < nh; ++q) {
                const double *tr = terms[q * (q - 1) / 2 + p];
                for (int k = 0; k < 3; ++k) aux[k] = __dadd_rn(aux[k], tr[k]);
            }
        double *out = E.pairs + ((size_t)s * 2 * kPairSlots + slot) * 3;
        out[0] = aux[0];
        out[1] = aux[1];
        out[2] = aux[2];
    }
}

// ---- Kepler drift -------------------------------------------------------------
// src/integrator_whfast.c:774-815
// Quotients x / d by the divisors d of the Stumpff series, correctly
// rounded without a division.  zh = RN(1/d) and zl = RN(1/d - zh) (exact
// rationals rounded once); q = RN(x zh + RN(x zl)) is within an ulp of x/d
// (Brisebarre, Muller and Raina, "Accelerating correctly rounded
// floating-point division when the divisor is known in advance", IEEE
// Trans. Computers 53(8), 2004), and one correction with the exact remainder
// r = x - q d gives RN(q + r zh) = RN(x/d) (Markstein, IBM J. Res. Dev.
// 34(1), 1990: a faithful quotient and a correctly rounded reciprocal).
// The remainder is exact while its last bit stays above the subnormal
// range, so |x| outside [2^-960, 2^960] (zeros, subnormals, infinities,
// NaN) takes the division itself.  Checked against __ddiv_rn bit for bit
// by gsgpu_stumpff_division_selftest.
struct StumpffDiv {
    double d, zh, zl;
};
enum { SD6, SD12, SD20, SD30, SD42, SD56, SD72, SD90, SD110, SD132, SD156, SD182, SD210, kStumpffDivs };
__constant__ StumpffDiv kStumpffDiv[kStumpffDivs] = {
    {6.0, 0x1.5555555555555p-3, 0x1.5555555555555p-57},
    {12.0, 0x1.5555555555555p-4, 0x1.5555555555555p-58},
    {20.0, 0x1.999999999999ap-5, -0x1.999999999999ap-59},
    {30.0, 0x1.1111111111111p-5, 0x1.1111111111111p-61},
    {42.0, 0x1.8618618618618p-6, 0x1.8618618618618p-60},
    {56.0, 0x1.2492492492492p-6, 0x1.2492492492492p-60},
    {72.0, 0x1.c71c71c71c71cp-7, 0x1.c71c71c71c71cp-61},
    {90.0, 0x1.6c16c16c16c17p-7, -0x1.f49f49f49f49fp-62},
    {110.0, 0x1.29e4129e4129ep-7, 0x1.04a7904a7904ap-61},
    {132.0, 0x1.f07c1f07c1f08p-8, -0x1.f07c1f07c1f08p-63},
    {156.0, 0x1.a41a41a41a41ap-8, 0x1.0690690690690p-62},
    {182.0, 0x1.6816816816817p-8, -0x1.fa5fa5fa5fa60p-62},
    {210.0, 0x1.3813813813814p-8, -0x1.fb1fb1fb1fb20p-62},
};

template <int K> __device__ __forceinline__ double sdiv(double x)
{
    const double d = kStumpffDiv[K].d, zh = kStumpffDiv[K].zh, zl = kStumpffDiv[K].zl;
    const double ax = fabs(x);
    if (!(ax >= 0x1p-960 && ax <= 0x1p+960)) return __ddiv_rn(x, d);
    const double q = __fma_rn(x, zh, __dmul_rn(x, zl));
    const double r = __fma_rn(-q, d, x);
    return __fma_rn(r, zh, q);
}

__device__ __forceinline__ void stumpff(double z, double &c0, double &c1, double &c2, double &c3)
{
    int q = 0;
    while (fabs(z) > 0.1) {
        z = __ddiv_rn(z, 4.0);
        ++q;
    }
    double t = __dsub_rn(1.0, sdiv<SD210>(z));
    t = __dsub_rn(1.0, __dmul_rn(sdiv<SD156>(z), t));
    t = __dsub_rn(1.0, __dmul_rn(sdiv<SD110>(z), t));
    t = __dsub_rn(1.0, __dmul_rn(sdiv<SD72>(z), t));
    t = __dsub_rn(1.0, __dmul_rn(sdiv<SD42>(z), t));
    t = __dsub_rn(1.0, __dmul_rn(sdiv<SD20>(z), t));
    double s3 = sdiv<SD6>(t);
    double u = __dsub_rn(1.0, sdiv<SD182>(z));
    u = __dsub_rn(1.0, __dmul_rn(sdiv<SD132>(z), u));
    u = __dsub_rn(1.0, __dmul_rn(sdiv<SD90>(z), u));
    u = __dsub_rn(1.0, __dmul_rn(sdiv<SD56>(z), u));
    u = __dsub_rn(1.0, __dmul_rn(sdiv<SD30>(z), u));
    u = __dsub_rn(1.0, __dmul_rn(sdiv<SD12>(z), u));
    double s2 = __dmul_rn(u, 0.5);   // u / 2, exact scaling: the same rounding
    double s1 = __dsub_rn(1.0, __dmul_rn(z, s3));
    double s0 = __dsub_rn(1.0, __dmul_rn(z, s2));
    while (q > 0) {
        s3 = __ddiv_rn(__dadd_rn(s2, __dmul_rn(s0, s3)), 4.0);
        s2 = __ddiv_rn(__dmul_rn(s1, s1), 2.0);
        s1 = __dmul_rn(s0, s1);
        s0 = __dsub_rn(__dmul_rn(__dmul_rn(2.0, s0), s0), 1.0);
        --q;
    }
    c0 = s0;
    c1 = s1;
    c2 = s2;
    c3 = s3;
}

// src/integrator_whfast.c:424-600 for one Jacobi body; returns true when the
// particle has to be removed.
__device__ bool kepler_drift(double *jx, double *jv, double gm, double dt)
{
    const double xx[3] = {jx[0], jx[1], jx[2]};
    const double vv[3] = {jv[0], jv[1], jv[2]};
    const double xn = norm3d(xx);
    const double vn = norm3d(vv);
    const double rv = __ddiv_rn(dot3(xx, vv), xn);
    const double alpha = __dsub_rn(__ddiv_rn(__dmul_rn(2.0, gm), xn), __dmul_rn(vn, vn));
    double s = __ddiv_rn(dt, xn);
    double c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0;
    bool conv = false, bad_z = false;
    const double xrv = __dmul_rn(xn, rv);
    for (int it = 0; it < 500; ++it) {
        const double ss = __dmul_rn(s, s);
        const double z = __dmul_rn(alpha, ss);
        if (!isfinite(z)) {
            bad_z = true;
            break;
        }
        stumpff(z, c0, c1, c2, c3);
        const double sss = __dmul_rn(ss, s);
        const double F = __dsub_rn(__dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(xn, s), c1),
                                                       __dmul_rn(__dmul_rn(xrv, ss), c2)),
                                             __dmul_rn(__dmul_rn(gm, sss), c3)),
                                   dt);
        const double dF = __dadd_rn(__dadd_rn(__dmul_rn(xn, c0), __dmul_rn(__dmul_rn(xrv, s), c1)),
                                    __dmul_rn(__dmul_rn(gm, ss), c2));
        const double ds = __ddiv_rn(-F, dF);
        s = __dadd_rn(s, ds);
        if (fabs(ds) < 1e-12) {
            conv = true;
            break;
        }
    }
    const double ss = __dmul_rn(s, s);
    const double sss = __dmul_rn(ss, s);
    const double r = __dadd_rn(__dadd_rn(__dmul_rn(xn, c0), __dmul_rn(__dmul_rn(xrv, s), c1)),
                               __dmul_rn(__dmul_rn(gm, ss), c2));
    bool remove = false;
    if (!conv) {
        const double F = __dsub_rn(__dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(xn, s), c1),
                                                       __dmul_rn(__dmul_rn(xrv, ss), c2)),
                                             __dmul_rn(__dmul_rn(gm, sss), c3)),
                                   dt);
        const double err = __ddiv_rn(F, r);
        remove = (err > 1e-5) || bad_z;
    }
    const double f = __dsub_rn(1.0, __ddiv_rn(__dmul_rn(__dmul_rn(gm, ss), c2), xn));
    const double g = __dsub_rn(dt, __dmul_rn(__dmul_rn(gm, sss), c3));
    const double df = __ddiv_rn(__dmul_rn(__dmul_rn(-gm, s), c1), __dmul_rn(r, xn));
    const double dg = __dsub_rn(1.0, __ddiv_rn(__dmul_rn(__dmul_rn(gm, ss), c2), r));
    for (int k = 0; k < 3; ++k) {
        jx[k] = __dadd_rn(__dmul_rn(f, xx[k]), __dmul_rn(g, vv[k]));
        jv[k] = __dadd_rn(__dmul_rn(df, xx[k]), __dmul_rn(dg, vv[k]));
    }
    return remove;
}

__global__ void k_wh_drift(EnsDev E, int P, double dt)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int s = E.sys_of[p];
    const int base = E.off[s];
    const int i = p - base;
    if (i == 0 || i >= E.cnt[s]) return;
    const double gm = __ddiv_rn(__dmul_rn(__dmul_rn(E.G, E.m[base]), E.eta[p]), E.eta[p - 1]);
    const bool rm = kepler_drift(E.jx + 3 * (size_t)p, E.jv + 3 * (size_t)p, gm, dt);
    if (rm && E.remove_invalid) {
        E.rm[p] = 1;
        atomicAdd(&E.nrm[s], 1);
    }
}

// ---- interaction accelerations ---------------------------------------------
// src/integrator_whfast.c:959-1264 (massless) / :839-957 (pairwise).
__global__ void k_wh_accel(EnsDev E, int P)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int s = E.sys_of[p];
    const int base = E.off[s];
    const int i = p - base;
    const int n = E.cnt[s];
    if (i >= n) return;
    double *a = E.a + 3 * (size_t)p;
    if (i == 0) {
        a[0] = a[1] = a[2] = 0.0;
        return;
    }
    const double *x = E.x + 3 * (size_t)base;
    const double *m = E.m + base;
    const double *eta = E.eta + base;
    const int *hv = E.hv + base;
    const int nh = E.nh[s];
    const double e3 = __dmul_rn(__dmul_rn(E.eps, E.eps), E.eps);
    const double G = E.G;
    const bool massive = (E.variant == WH_PAIRWISE) || m[i] != 0.0;
    const double xi[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
    const double tv[3] = {__dsub_rn(xi[0], x[0]), __dsub_rn(xi[1], x[1]), __dsub_rn(xi[2], x[2])};
    const double tn = norm3d(tv);
    const double tc = __dadd_rn(__dmul_rn(__dmul_rn(tn, tn), tn), e3);
    const double *jxi = E.jx + 3 * (size_t)p;
    const double jn = norm3d(jxi);
    const double jc = __dadd_rn(__dmul_rn(__dmul_rn(jn, jn), jn), e3);
    const double Gm0 = __dmul_rn(G, m[0]);
    const double pre = massive ? __ddiv_rn(__dmul_rn(Gm0, eta[i]), eta[i - 1]) : Gm0;
    double acc[3];
    for (int k = 0; k < 3; ++k)
        acc[k] = __dmul_rn(pre, __dsub_rn(__ddiv_rn(jxi[k], jc), __ddiv_rn(tv[k], tc)));
    double aux[3] = {0.0, 0.0, 0.0};
    for (int q = 1; q < nh; ++q) {
        const int j = hv[q];
        if (j >= i) break;
        const double d[3] = {__dsub_rn(xi[0], x[3 * j]), __dsub_rn(xi[1], x[3 * j + 1]),
                             __dsub_rn(xi[2], x[3 * j + 2])};
        const double dn = norm3d(d);
        const double dc = __dadd_rn(__dmul_rn(__dmul_rn(dn, dn), dn), e3);
        const double Gm = __dmul_rn(G, m[j]);
        for (int k = 0; k < 3; ++k) aux[k] = __dadd_rn(aux[k], __ddiv_rn(__dmul_rn(Gm, d[k]), dc));
    }
    for (int k = 0; k < 3; ++k)
        acc[k] = __dsub_rn(acc[k],
                           massive ? __ddiv_rn(__dmul_rn(aux[k], eta[i]), eta[i - 1]) : aux[k]);
    aux[0] = aux[1] = aux[2] = 0.0;
    for (int q = 1; q < nh; ++q) {
        const int j = hv[q];
        if (j <= i) continue;
        const double d[3] = {__dsub_rn(x[3 * j], xi[0]), __dsub_rn(x[3 * j + 1], xi[1]),
                             __dsub_rn(x[3 * j + 2], xi[2])};
        const double dn = norm3d(d);
        const double dc = __dadd_rn(__dmul_rn(__dmul_rn(dn, dn), dn), e3);
        const double Gm = __dmul_rn(G, m[j]);
        for (int k = 0; k < 3; ++k) aux[k] = __dadd_rn(aux[k], __ddiv_rn(__dmul_rn(Gm, d[k]), dc));
    }
    for (int k = 0; k < 3; ++k) acc[k] = __dadd_rn(acc[k], aux[k]);
    aux[0] = aux[1] = aux[2] = 0.0;
    if (nh <= kPairMax) {
        int g = 0, rank = -1;
        for (int q = 0; q < nh; ++q) {
            const int j = hv[q];
            if (j == i) rank = q;
            if (j < i) ++g;
        }
        const int slot = rank >= 0 ? kPairSlots + rank : g;
        const double *pr = E.pairs + ((size_t)s * 2 * kPairSlots + slot) * 3;
        for (int k = 0; k < 3; ++k) a[k] = __dsub_rn(acc[k], __ddiv_rn(pr[k], eta[i - 1]));
        return;
    }
    for (int q0 = 0; q0 < nh; ++q0) {
        const int j = hv[q0];
        if (j >= i) break;
        const double Gmj = __dmul_rn(G, m[j]);
        for (int q1 = q0 + 1; q1 < nh; ++q1) {
            const int kk = hv[q1];
            if (kk <= i) continue;
            const double d[3] = {__dsub_rn(x[3 * kk], x[3 * j]), __dsub_rn(x[3 * kk + 1], x[3 * j + 1]),
                                 __dsub_rn(x[3 * kk + 2], x[3 * j + 2])};
            const double dn = norm3d(d);
            const double dc = __dadd_rn(__dmul_rn(__dmul_rn(dn, dn), dn), e3);
            const double Gmm = __dmul_rn(Gmj, m[kk]);
            for (int k = 0; k < 3; ++k)
                aux[k] = __dadd_rn(aux[k], __ddiv_rn(__dmul_rn(Gmm, d[k]), dc));
        }
    }
    for (int k = 0; k < 3; ++k) a[k] = __dsub_rn(acc[k], __ddiv_rn(aux[k], eta[i - 1]));
}

__global__ void k_wh_kick(EnsDev E, int P, double h)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int s = E.sys_of[p];
    if (p - E.off[s] >= E.cnt[s]) return;
    for (int k = 0; k < 3; ++k)
        E.jv[3 * (size_t)p + k] = __dadd_rn(E.jv[3 * (size_t)p + k], __dmul_rn(E.a[3 * (size_t)p + k], h));
}

// ---- leapfrog + massless acceleration (src/acceleration.c:236-367) ---------
__global__ void k_ens_massless_accel(EnsDev E, int P)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int s = E.sys_of[p];
    const int base = E.off[s];
    const int i = p - base;
    const int n = E.cnt[s];
    if (i >= n) return;
    const double *x = E.x + 3 * (size_t)base;
    const double *m = E.m + base;
    const int *hv = E.hv + base;
    const int nh = E.nh[s];
    const double eps2 = __dmul_rn(E.eps, E.eps);
    const double xi0 = x[3 * i], xi1 = x[3 * i + 1], xi2 = x[3 * i + 2];
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    // the pairwise variant lists every particle and is the symmetric sum of
    // src/acceleration.c:177-234 seen from particle i (same term order)
    if (E.variant == WH_PAIRWISE || m[i] != 0.0) {
        for (int q = 0; q < nh; ++q) {
            const int j = hv[q];
            if (j == i) continue;
            const double r0 = __dsub_rn(xi0, x[3 * j]), r1 = __dsub_rn(xi1, x[3 * j + 1]),
                         r2 = __dsub_rn(xi2, x[3 * j + 2]);
            const double rn = __dsqrt_rn(__dadd_rn(
                __dadd_rn(__dadd_rn(__dmul_rn(r0, r0), __dmul_rn(r1, r1)), __dmul_rn(r2, r2)), eps2));
            const double t = __ddiv_rn(E.G, __dmul_rn(__dmul_rn(rn, rn), rn));
            const double mj = m[j];
            a0 = __dsub_rn(a0, __dmul_rn(__dmul_rn(t, r0), mj));
            a1 = __dsub_rn(a1, __dmul_rn(__dmul_rn(t, r1), mj));
            a2 = __dsub_rn(a2, __dmul_rn(__dmul_rn(t, r2), mj));
        }
    } else {
        for (int q = 0; q < nh; ++q) {
            const int j = hv[q];
            const double r0 = __dsub_rn(x[3 * j], xi0), r1 = __dsub_rn(x[3 * j + 1], xi1),
                         r2 = __dsub_rn(x[3 * j + 2], xi2);
            const double rn = __dsqrt_rn(__dadd_rn(
                __dadd_rn(__dadd_rn(__dmul_rn(r0, r0), __dmul_rn(r1, r1)), __dmul_rn(r2, r2)), eps2));
            const double t = __ddiv_rn(E.G, __dmul_rn(__dmul_rn(rn, rn), rn));
            const double mq = m[q];   // the reference's loop-index mass read
            a0 = __dadd_rn(a0, __dmul_rn(__dmul_rn(t, r0), mq));
            a1 = __dadd_rn(a1, __dmul_rn(__dmul_rn(t, r1), mq));
            a2 = __dadd_rn(a2, __dmul_rn(__dmul_rn(t, r2), mq));
        }
    }
    E.a[3 * (size_t)p] = a0;
    E.a[3 * (size_t)p + 1] = a1;
    E.a[3 * (size_t)p + 2] = a2;
}

__global__ void __launch_bounds__(32 * SEQ_WARPS) k_ens_massive_list(EnsDev E)
{
    const int s = blockIdx.x * SEQ_WARPS + (threadIdx.x >> 5);
    if (s >= E.S) return;   // warp-uniform
    wh_massive_list_warp(E, E.off[s], E.cnt[s], s, threadIdx.x & 31);
}

// Self-check of sdiv against the division it replaces: sample k of the
// n checked per divisor is a 64-bit pattern (every exponent, subnormals,
// infinities, NaN) for even k, and for odd k a dividend whose exact
// quotient lies halfway between two doubles (the hardest rounding case).
__device__ __forceinline__ unsigned long long mix64(unsigned long long z)
{
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

template <int K> __device__ bool sdiv_matches(double x)
{
    const double a = sdiv<K>(x), b = __ddiv_rn(x, kStumpffDiv[K].d);
    return (isnan(a) && isnan(b)) || __double_as_longlong(a) == __double_as_longlong(b);
}

__global__ void k_sdiv_selftest(long long n, unsigned long long seed, unsigned long long *bad)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    unsigned long long local = 0;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += stride) {
        const unsigned long long h = mix64(seed ^ mix64((unsigned long long)k));
        double x;
        const int which = (int)(h % kStumpffDivs);
        if (k & 1) {
            // x = RN((q0 + ulp(q0) / 2) d): the exact quotient x / d lies
            // next to the midpoint of two neighbouring doubles
            const unsigned long long m = (mix64(h) >> 11) | (1ull << 52);
            const int e = (int)(mix64(h + 1) % 241) - 120;
            const double q0 = scalbn((double)m, e - 52);
            const double half_ulp_d = __dmul_rn(scalbn(1.0, e - 53), kStumpffDiv[which].d);
            x = __fma_rn(q0, kStumpffDiv[which].d, half_ulp_d);
        } else {
            x = __longlong_as_double((long long)h);
        }
        bool ok = true;
        switch (which) {
        case SD6: ok = sdiv_matches<SD6>(x); break;
        case SD12: ok = sdiv_matches<SD12>(x); break;
        case SD20: ok = sdiv_matches<SD20>(x); break;
        case SD30: ok = sdiv_matches<SD30>(x); break;
        case SD42: ok = sdiv_matches<SD42>(x); break;
        case SD56: ok = sdiv_matches<SD56>(x); break;
        case SD72: ok = sdiv_matches<SD72>(x); break;
        case SD90: ok = sdiv_matches<SD90>(x); break;
        case SD110: ok = sdiv_matches<SD110>(x); break;
        case SD132: ok = sdiv_matches<SD132>(x); break;
        case SD156: ok = sdiv_matches<SD156>(x); break;
        case SD182: ok = sdiv_matches<SD182>(x); break;
        default: ok = sdiv_matches<SD210>(x); break;
        }
        local += ok ? 0 : 1;
    }
    if (local) atomicAdd(bad, local);
}

}  // namespace gs

// Checks the division-free Stumpff quotients against __ddiv_rn on n
// samples; *mismatches receives the count of differing results.
extern "C" int gsgpu_stumpff_division_selftest(long long n, unsigned long long seed,
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
        gs::k_sdiv_selftest<<<1216, 256>>>(n, seed, bad.as<unsigned long long>());
        e = cudaGetLastError();
    }
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, bad.p, sizeof(h), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        std::fprintf(stderr, "gsgpu_stumpff_division_selftest: %s\n", cudaGetErrorString(e));
        return GRAV_FAILURE;
    }
    *mismatches = (long long)h;
    return GRAV_SUCCESS;
}

// ---------------------------------------------------------------------------
// Host side: the ensemble object.
// ---------------------------------------------------------------------------
using namespace gs;

// The sort is launched once per size class of systems, with shared memory
// and threads for the largest system of the class, so that the many small
// systems do not each reserve the largest system's shared memory.
constexpr int kSortClasses = 3;
constexpr int kSortClassPow2[kSortClasses] = {256, 1024, kEnsembleMaxSystem};

struct gsgpu_ensemble {
    int S = 0, P = 0, max_n = 0, pow2 = 1;
    DBuf sort_list;                        // system ids grouped by class
    int sort_first[kSortClasses + 1] = {};  // class c: sort_list[sort_first[c]..sort_first[c+1])
    int sort_pow2[kSortClasses] = {};       // largest power of two of the class's systems
    int integrator = INTEGRATOR_WHFAST;
    double dt = 0.0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::vector<int> h_off;
    DBuf off, cnt, sys_of, ids, x, v, m, jx, jv, a, eta, hv, nh, rm, nrm, t_ids, t_x, t_v, t_m,
        status, xe, ve, pairs, seq_nmass, seq_runs, run_lo, run_hi, run_y;
    EnsDev E{};
    bool primed = false;
    double last_dt = 0.0;
    cudaGraphExec_t graph = nullptr;
    double graph_dt = 0.0;
    // Kernel timing (gsgpu_ensemble_set_kernel_timing): steps launch
    // directly, with CUDA events around the drift and around the
    // interaction accelerations (pair sums + per-particle terms).
    bool timing = false;
    ForceTimer t_drift, t_accel;

    ~gsgpu_ensemble()
    {
        if (graph) cudaGraphExecDestroy(graph);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }

    int pgrid() const { return (P + 127) / 128; }
    int tpb_accel = 128, tpb_drift = 128;   // chosen by autotune()
    // threads per system of the sort, per size class (0: the class's default,
    // half its largest system's power of two); chosen by autotune()
    int sort_tpb[kSortClasses] = {0, 0, 0};
    bool tuned = false;
    int grid_for(int t) const { return (P + t - 1) / t; }

    // Thread-block sizes of the per-particle kernels, timed once on this
    // ensemble right after its first half kick (before any graph capture).
    // Only launches that leave the simulation unchanged are timed: the
    // accelerations are recomputed from the same positions, and the drift
    // runs on scratch copies of the Jacobi arrays with removals off.
    ErrorStatus autotune()
    {
        if (tuned) return ok();
        tuned = true;
        const int cand[4] = {64, 128, 256, 512};
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        GS_CUDA(cudaEventCreate(&e0));
        GS_CUDA(cudaEventCreate(&e1));
        ErrorStatus st = ok();
        auto best_of = [&](auto launch, int &choice) {
            float best = 1e30f;
            for (int t : cand) {
                launch(t);
                if (cudaEventRecord(e0, stream) != cudaSuccess) break;
                launch(t);
                launch(t);
                if (cudaEventRecord(e1, stream) != cudaSuccess) break;
                if (cudaEventSynchronize(e1) != cudaSuccess) break;
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < best) {
                    best = ms;
                    choice = t;
                }
            }
        };
        if (integrator == INTEGRATOR_WHFAST) {
            best_of([&](int t) { k_wh_accel<<<grid_for(t), t, 0, stream>>>(E, P); }, tpb_accel);
            EnsDev Es = E;
            Es.jx = E.t_x;
            Es.jv = E.t_v;
            Es.remove_invalid = 0;
            cudaMemcpyAsync(E.t_x, E.jx, (size_t)P * 3 * sizeof(double), cudaMemcpyDeviceToDevice,
                            stream);
            cudaMemcpyAsync(E.t_v, E.jv, (size_t)P * 3 * sizeof(double), cudaMemcpyDeviceToDevice,
                            stream);
            best_of([&](int t) { k_wh_drift<<<grid_for(t), t, 0, stream>>>(Es, P, dt); },
                    tpb_drift);
            // Threads per system of the sort by distance, per size class.  The
            // step starts with this sort of the Jacobi arrays, and sorting them
            // again finds them in order, so these launches leave the step's
            // result unchanged.
            for (int c = 0; c < kSortClasses; ++c) {
                const int count = sort_first[c + 1] - sort_first[c];
                if (count == 0) continue;
                const int p2 = sort_pow2[c];
                float best = 1e30f;
                for (int div : {2, 4, 8, 16}) {
                    const int t = std::min(1024, std::max(32, p2 / div));
                    auto launch = [&]() {
                        k_wh_sort<<<count, t, (size_t)p2 * 12, stream>>>(
                            E, E.jx, E.jv, p2, 0, sort_list.as<int>() + sort_first[c]);
                    };
                    launch();
                    if (cudaEventRecord(e0, stream) != cudaSuccess) break;
                    launch();
                    launch();
                    if (cudaEventRecord(e1, stream) != cudaSuccess) break;
                    if (cudaEventSynchronize(e1) != cudaSuccess) break;
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (ms < best) {
                        best = ms;
                        sort_tpb[c] = t;
                    }
                }
            }
        } else {
            best_of([&](int t) { k_ens_massless_accel<<<grid_for(t), t, 0, stream>>>(E, P); },
                    tpb_accel);
        }
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) st = GS_RAISE(GRAV_FAILURE, "ensemble autotune: %s", cudaGetErrorString(e));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return st;
    }

    ErrorStatus sort(double *vec, double *vel)
    {
        for (int c = 0; c < kSortClasses; ++c) {
            const int count = sort_first[c + 1] - sort_first[c];
            if (count == 0) continue;
            const int p2 = sort_pow2[c];
            const size_t smem = (size_t)p2 * 12;
            // one thread per pair of slots for the odd-even passes, 32..1024,
            // unless the autotuner chose fewer
            const int threads = sort_tpb[c] > 0 ? sort_tpb[c] : std::min(1024, std::max(32, p2 / 2));
            k_wh_sort<<<count, threads, smem, stream>>>(E, vec, vel, p2, vec == E.x ? 1 : 0,
                                                        sort_list.as<int>() + sort_first[c]);
        }
        GS_CUDA(cudaGetLastError());
        return ok();
    }

    int seq_grid() const { return (S + SEQ_WARPS - 1) / SEQ_WARPS; }

    // Removals, eta and Jacobi -> Cartesian (src/integrator_whfast.c:726-772)
    ErrorStatus to_cartesian(const EnsDev &D)
    {
        k_wh_seq_scan<<<S, SCAN_THREADS, 0, stream>>>(D);
        k_wh_seq_chain<<<(S + 63) / 64, 64, 0, stream>>>(D);
        k_wh_seq_fill<<<pgrid(), 128, 0, stream>>>(D, P);
        GS_CUDA(cudaGetLastError());
        return ok();
    }

    ErrorStatus accel(ForceTimer *timer = nullptr)
    {
        if (timer) GS_TRY(timer->begin(stream));
        if (integrator == INTEGRATOR_WHFAST) {
            k_wh_pairs<<<(S + PAIR_WARPS - 1) / PAIR_WARPS, 32 * PAIR_WARPS, 0, stream>>>(E);
            k_wh_accel<<<grid_for(tpb_accel), tpb_accel, 0, stream>>>(E, P);
        }
        else
            k_ens_massless_accel<<<grid_for(tpb_accel), tpb_accel, 0, stream>>>(E, P);
        if (timer) GS_TRY(timer->end(stream));
        GS_CUDA(cudaGetLastError());
        return ok();
    }

    ErrorStatus prime(OutputContext *oc = nullptr, const SimulationStatus *status = nullptr)
    {
        if (primed) return ok();
        if (integrator == INTEGRATOR_WHFAST) {
            // src/integrator_whfast.c:241-273
            GS_TRY(sort(E.x, E.v));
            if (oc && oc->initial()) {
                // the initial snapshot is of the system sorted by distance
                GS_TRY(snapshot(oc, E.v, status ? status->t : 0.0, status ? status->dt : 0.0));
            }
            k_wh_seq_init<<<seq_grid(), 32 * SEQ_WARPS, 0, stream>>>(E);
            GS_TRY(accel());
            k_wh_kick<<<pgrid(), 128, 0, stream>>>(E, P, 0.5 * dt);
        } else {
            k_ens_massive_list<<<seq_grid(), 32 * SEQ_WARPS, 0, stream>>>(E);
            GS_TRY(accel());
            launch_comp_update(E.v, ve.as<double>(), E.a, dt, 0.5, 3 * P, stream);
        }
        GS_CUDA(cudaGetLastError());
        primed = true;
        GS_TRY(autotune());
        return ok();
    }

    ErrorStatus step(double h)
    {
        ForceTimer *td = timing ? &t_drift : nullptr, *ta = timing ? &t_accel : nullptr;
        if (integrator == INTEGRATOR_WHFAST) {
            // src/integrator_whfast.c:290-343
            GS_TRY(sort(E.jx, E.jv));
            if (td) GS_TRY(td->begin(stream));
            k_wh_drift<<<grid_for(tpb_drift), tpb_drift, 0, stream>>>(E, P, h);
            if (td) GS_TRY(td->end(stream));
            GS_TRY(to_cartesian(E));
            GS_TRY(accel(ta));
            k_wh_kick<<<pgrid(), 128, 0, stream>>>(E, P, h);
        } else {
            launch_comp_update(E.x, xe.as<double>(), E.v, h, 1.0, 3 * P, stream);
            GS_TRY(accel(ta));
            launch_comp_update(E.v, ve.as<double>(), E.a, h, 1.0, 3 * P, stream);
        }
        GS_CUDA(cudaGetLastError());
        last_dt = h;
        return ok();
    }

    int sort_launches() const
    {
        int k = 0;
        for (int c = 0; c < kSortClasses; ++c) k += sort_first[c + 1] > sort_first[c] ? 1 : 0;
        return k;
    }
    int kernels_per_step() const { return integrator == INTEGRATOR_WHFAST ? 7 + sort_launches() : 3; }

    // Snapshot of system 0 (a launch_simulation run holds one system): E.x
    // and the velocity array dv with the ids and masses of its live slots.
    ErrorStatus snapshot(OutputContext *oc, const double *dv, double t, double h)
    {
        return oc->take(P, E.x, dv, E.ids, E.m, E.cnt, stream, t, h);
    }

    // src/integrator_whfast.c:345-364: the Cartesian state at integer time
    // from the Jacobi velocities kicked back by half a step (in scratch),
    // written into the Cartesian arrays, which the next step recomputes.
    ErrorStatus whfast_snapshot(OutputContext *oc, double t, double h)
    {
        GS_CUDA(cudaMemcpyAsync(E.t_v, E.jv, (size_t)P * 3 * sizeof(double),
                                cudaMemcpyDeviceToDevice, stream));
        EnsDev T = E;
        T.jv = E.t_v;
        k_wh_kick<<<pgrid(), 128, 0, stream>>>(T, P, -0.5 * h);
        GS_TRY(to_cartesian(T));
        GS_CUDA(cudaGetLastError());
        return snapshot(oc, E.v, t, h);
    }

    ErrorStatus step_graph(double h)
    {
        if (timing) {
            GS_TRY(step(h));
            GS_TRY(t_drift.collect());
            GS_TRY(t_accel.collect());
            return ok();
        }
        if (!graph || graph_dt != h) {
            if (graph) {
                cudaGraphExecDestroy(graph);
                graph = nullptr;
            }
            cudaGraph_t g = nullptr;
            GS_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            ErrorStatus st = step(h);
            cudaError_t e = cudaStreamEndCapture(stream, &g);
            if (st.return_code != GRAV_SUCCESS) {
                if (g) cudaGraphDestroy(g);
                return st;
            }
            if (e != cudaSuccess) {
                (void)cudaGetLastError();
                return step(h);
            }
            e = cudaGraphInstantiate(&graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                (void)cudaGetLastError();
                graph = nullptr;
                return step(h);
            }
            graph_dt = h;
        }
        GS_CUDA(cudaGraphLaunch(graph, stream));
        last_dt = h;
        return ok();
    }

    ErrorStatus check()
    {
        unsigned h = 0;
        GS_CUDA(cudaMemcpyAsync(&h, status.p, sizeof(h), cudaMemcpyDeviceToHost, stream));
        GS_CUDA(cudaStreamSynchronize(stream));
        if (h & ST_CAPACITY)
            return GS_RAISE(GRAV_VALUE_ERROR, "a system exceeds the ensemble's sort capacity");
        if (h & ST_NONFINITE)
            return GS_RAISE(GRAV_VALUE_ERROR, "an ensemble sort saw an inconsistent order");
        if (h & ST_NO_PRIMARY)
            return GS_RAISE(GRAV_VALUE_ERROR, "Primary particle ID not found in system");
        return ok();
    }
};

namespace gs {

ErrorStatus ensemble_create(gsgpu_ensemble **out, int num_systems, const int *counts, double G,
                            int integrator, int method, double eps, double dt,
                            int remove_invalid, cudaStream_t stream)
{
    if (!out || !counts) return GS_RAISE(GRAV_POINTER_ERROR, "NULL argument");
    if (num_systems <= 0) return GS_RAISE(GRAV_VALUE_ERROR, "num_systems must be positive");
    if (!(dt > 0.0)) return GS_RAISE(GRAV_VALUE_ERROR, "dt must be positive. Got: %g", dt);
    if (integrator != INTEGRATOR_WHFAST && integrator != INTEGRATOR_LEAPFROG)
        return GS_RAISE(GRAV_VALUE_ERROR, "ensembles run WHFast (10) or leapfrog (4). Got: %d",
                        integrator);
    if (method != GRAV_GPU_MASSLESS && method != GRAV_GPU_PAIRWISE &&
        method != GRAV_GPU_PAIRWISE_FP64)
        return GS_RAISE(GRAV_VALUE_ERROR,
                        "Invalid acceleration method for WHFast integrator. Only pairwise and "
                        "massless methods are supported.");
    const DeviceInfo *d = nullptr;
    GS_TRY(device_info(&d));
    std::unique_ptr<gsgpu_ensemble> e(new gsgpu_ensemble());
    e->S = num_systems;
    e->integrator = integrator;
    e->dt = dt;
    long long total = 0;
    for (int s = 0; s < num_systems; ++s) total += counts[s] > 0 ? counts[s] : 0;
    if (total > kMaxParticles)
        return GS_RAISE(GRAV_VALUE_ERROR, "ensemble of %lld particles exceeds %d", total,
                        kMaxParticles);
    e->h_off.assign(num_systems + 1, 0);
    for (int s = 0; s < num_systems; ++s) {
        if (counts[s] <= 0) return GS_RAISE(GRAV_VALUE_ERROR, "system %d is empty", s);
        e->h_off[s + 1] = e->h_off[s] + counts[s];
        e->max_n = std::max(e->max_n, counts[s]);
    }
    e->P = e->h_off[num_systems];
    while (e->pow2 < e->max_n) e->pow2 <<= 1;
    if (e->pow2 > kEnsembleMaxSystem)
        return GS_RAISE(GRAV_VALUE_ERROR, "systems of more than %d particles are not supported",
                        kEnsembleMaxSystem);
    if (stream) {
        e->stream = stream;
    } else {
        GS_CUDA(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
        e->own_stream = true;
    }
    const size_t P = (size_t)e->P, S = (size_t)e->S;
    GS_TRY(e->off.reserve((S + 1) * sizeof(int)));
    GS_TRY(e->cnt.reserve(S * sizeof(int)));
    GS_TRY(e->nh.reserve(S * sizeof(int)));
    GS_TRY(e->nrm.reserve(S * sizeof(int)));
    DBuf *ints[] = {&e->sys_of, &e->ids, &e->hv, &e->rm, &e->t_ids};
    for (DBuf *b : ints) GS_TRY(b->reserve(P * sizeof(int)));
    DBuf *vec3[] = {&e->x, &e->v, &e->jx, &e->jv, &e->a, &e->t_x, &e->t_v, &e->xe, &e->ve};
    for (DBuf *b : vec3) GS_TRY(b->reserve(P * 3 * sizeof(double)));
    GS_TRY(e->m.reserve(P * sizeof(double)));
    GS_TRY(e->eta.reserve(P * sizeof(double)));
    GS_TRY(e->t_m.reserve(P * sizeof(double)));
    GS_TRY(e->status.reserve(sizeof(unsigned)));
    GS_TRY(e->seq_nmass.reserve(S * sizeof(int)));
    GS_TRY(e->seq_runs.reserve(S * sizeof(int)));
    GS_TRY(e->run_lo.reserve(S * (kSeqMassMax + 1) * sizeof(int)));
    GS_TRY(e->run_hi.reserve(S * (kSeqMassMax + 1) * sizeof(int)));
    GS_TRY(e->run_y.reserve(S * (kSeqMassMax + 1) * 6 * sizeof(double)));
    GS_TRY(e->pairs.reserve(S * 2 * kPairSlots * 3 * sizeof(double)));
    std::vector<int> sys(P);
    for (int s = 0; s < num_systems; ++s)
        for (int p = e->h_off[s]; p < e->h_off[s + 1]; ++p) sys[p] = s;
    GS_CUDA(cudaMemcpy(e->off.p, e->h_off.data(), (S + 1) * sizeof(int), cudaMemcpyHostToDevice));
    GS_CUDA(cudaMemcpy(e->cnt.p, counts, S * sizeof(int), cudaMemcpyHostToDevice));
    GS_CUDA(cudaMemcpy(e->sys_of.p, sys.data(), P * sizeof(int), cudaMemcpyHostToDevice));
    GS_CUDA(cudaMemset(e->nrm.p, 0, S * sizeof(int)));
    GS_CUDA(cudaMemset(e->rm.p, 0, P * sizeof(int)));
    GS_CUDA(cudaMemset(e->status.p, 0, sizeof(unsigned)));
    GS_CUDA(cudaMemset(e->a.p, 0, P * 3 * sizeof(double)));
    GS_CUDA(cudaFuncSetAttribute(k_wh_sort, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)std::max<size_t>((size_t)e->pow2 * 12, 48 * 1024)));
    {
        // size classes of the sort (counts only shrink, by removals)
        std::vector<int> list;
        list.reserve(S);
        for (int c = 0; c < kSortClasses; ++c) {
            e->sort_first[c] = (int)list.size();
            const int lo = c == 0 ? 0 : kSortClassPow2[c - 1];
            int p2 = 1;
            for (int s = 0; s < (int)S; ++s) {
                int q = 1;
                while (q < counts[s]) q <<= 1;
                if (q > lo && q <= kSortClassPow2[c]) {
                    list.push_back(s);
                    p2 = std::max(p2, q);
                }
            }
            e->sort_pow2[c] = p2;
        }
        e->sort_first[kSortClasses] = (int)list.size();
        GS_TRY(e->sort_list.reserve(list.size() * sizeof(int)));
        GS_CUDA(cudaMemcpy(e->sort_list.p, list.data(), list.size() * sizeof(int),
                           cudaMemcpyHostToDevice));
    }
    EnsDev &E = e->E;
    E.S = e->S;
    E.off = e->off.as<int>();
    E.cnt = e->cnt.as<int>();
    E.sys_of = e->sys_of.as<int>();
    E.ids = e->ids.as<int>();
    E.x = e->x.as<double>();
    E.v = e->v.as<double>();
    E.m = e->m.as<double>();
    E.jx = e->jx.as<double>();
    E.jv = e->jv.as<double>();
    E.a = e->a.as<double>();
    E.eta = e->eta.as<double>();
    E.hv = e->hv.as<int>();
    E.nh = e->nh.as<int>();
    E.rm = e->rm.as<int>();
    E.nrm = e->nrm.as<int>();
    E.t_ids = e->t_ids.as<int>();
    E.t_x = e->t_x.as<double>();
    E.t_v = e->t_v.as<double>();
    E.t_m = e->t_m.as<double>();
    E.status = e->status.as<unsigned>();
    E.pairs = e->pairs.as<double>();
    E.seq_nmass = e->seq_nmass.as<int>();
    E.seq_runs = e->seq_runs.as<int>();
    E.run_lo = e->run_lo.as<int>();
    E.run_hi = e->run_hi.as<int>();
    E.run_y = e->run_y.as<double>();
    E.G = G;
    E.eps = eps;
    E.variant = method == GRAV_GPU_MASSLESS ? WH_MASSLESS : WH_PAIRWISE;
    E.remove_invalid = remove_invalid ? 1 : 0;
    *out = e.release();
    return ok();
}

ErrorStatus ensemble_upload(gsgpu_ensemble *e, const int *ids, const double *x, const double *v,
                            const double *m)
{
    if (!e || !ids || !x || !v || !m) return GS_RAISE(GRAV_POINTER_ERROR, "NULL argument");
    const size_t P = (size_t)e->P;
    GS_CUDA(cudaMemcpyAsync(e->ids.p, ids, P * sizeof(int), cudaMemcpyHostToDevice, e->stream));
    GS_CUDA(cudaMemcpyAsync(e->x.p, x, P * 3 * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    GS_CUDA(cudaMemcpyAsync(e->v.p, v, P * 3 * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    GS_CUDA(cudaMemcpyAsync(e->m.p, m, P * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    GS_CUDA(cudaMemsetAsync(e->xe.p, 0, P * 3 * sizeof(double), e->stream));
    GS_CUDA(cudaMemsetAsync(e->ve.p, 0, P * 3 * sizeof(double), e->stream));
    e->primed = false;
    return ok();
}

// The reference's step loop over time tf (same step count and dt clamp).
ErrorStatus ensemble_run_until(gsgpu_ensemble *e, double tf, SimulationStatus *status,
                               const bool *is_exit, OutputContext *out)
{
    OutputContext *oc = out && out->active() ? out : nullptr;
    if (oc && (e->S != 1 || e->integrator != INTEGRATOR_WHFAST))
        return GS_RAISE(GRAV_VALUE_ERROR, "snapshots are written for one-system WHFast runs only");
    double dt = e->dt;
    const int64_t total = (int64_t)std::ceil(tf / dt);
    GS_TRY(e->prime(oc, status));
    if (oc) oc->begin();   // the initial snapshot leaves the next output time alone
    double t = 0.0;
    int64_t steps = 0;
    if (status) {
        status->t = 0.0;
        status->dt = dt;
        status->num_steps = 0;
    }
    while (steps < total) {
        if (t + dt > tf) dt = tf - t;
        if (status) status->dt = dt;
        GS_TRY(e->step_graph(dt));
        ++steps;
        t = (double)steps * dt;
        if (oc && oc->due(t)) GS_TRY(e->whfast_snapshot(oc, t, dt));
        if ((steps & 31) == 0) GS_TRY(e->check());
        if (is_exit && *is_exit) break;
    }
    if (status) {
        status->t = t;
        status->num_steps = steps;
    }
    GS_TRY(e->check());
    if (oc) GS_TRY(oc->finish());
    return ok();
}

// Final state: WHFast returns the Cartesian arrays as the reference leaves
// them; leapfrog synchronises v to integer time (src/integrator.c:1088-1094).
ErrorStatus ensemble_download(gsgpu_ensemble *e, int *counts, int *ids, double *x, double *v,
                              double *m)
{
    GS_TRY(e->check());
    const size_t P = (size_t)e->P;
    double *vsrc = e->E.v;
    if (e->integrator == INTEGRATOR_LEAPFROG && e->primed && v) {
        // v at integer time from the half-step state, without touching it
        GS_CUDA(cudaMemcpyAsync(e->t_v.p, e->v.p, P * 3 * sizeof(double), cudaMemcpyDeviceToDevice,
                                e->stream));
        launch_plain_kick(e->E.t_v, e->E.a, 0.5, e->last_dt, 3 * e->P, e->stream);
        GS_CUDA(cudaGetLastError());
        vsrc = e->E.t_v;
    }
    if (counts) GS_CUDA(cudaMemcpyAsync(counts, e->cnt.p, e->S * sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    if (ids) GS_CUDA(cudaMemcpyAsync(ids, e->ids.p, P * sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    if (x) GS_CUDA(cudaMemcpyAsync(x, e->x.p, P * 3 * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    if (v) GS_CUDA(cudaMemcpyAsync(v, vsrc, P * 3 * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    if (m) GS_CUDA(cudaMemcpyAsync(m, e->m.p, P * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    GS_CUDA(cudaStreamSynchronize(e->stream));
    return ok();
}

void ensemble_destroy(gsgpu_ensemble *e) { delete e; }

}  // namespace gs

extern "C" {

int gsgpu_ensemble_create(gsgpu_ensemble **out, int num_systems, const int *counts, double G,
                          int integrator, int acceleration_method, double softening_length,
                          double dt, int remove_invalid_particles, void *stream)
{
    ErrorStatus st = gs::ensemble_create(out, num_systems, counts, G, integrator, acceleration_method,
                                         softening_length, dt, remove_invalid_particles,
                                         static_cast<cudaStream_t>(stream));
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return 0;
}

int gsgpu_ensemble_upload(gsgpu_ensemble *e, const int *ids, const double *x, const double *v,
                          const double *m)
{
    ErrorStatus st = gs::ensemble_upload(e, ids, x, v, m);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return 0;
}

int gsgpu_ensemble_run(gsgpu_ensemble *e, int64_t num_steps)
{
    if (!e) return GRAV_POINTER_ERROR;
    ErrorStatus st = e->prime();
    for (int64_t k = 0; k < num_steps && st.return_code == GRAV_SUCCESS; ++k)
        st = e->step_graph(e->dt);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return 0;
}

int gsgpu_ensemble_run_until(gsgpu_ensemble *e, double tf)
{
    if (!e) return GRAV_POINTER_ERROR;
    ErrorStatus st = gs::ensemble_run_until(e, tf, nullptr, nullptr);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return 0;
}

int gsgpu_ensemble_download(gsgpu_ensemble *e, int *counts, int *ids, double *x, double *v,
                            double *m)
{
    if (!e) return GRAV_POINTER_ERROR;
    ErrorStatus st = gs::ensemble_download(e, counts, ids, x, v, m);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return 0;
}

int gsgpu_ensemble_kernels_per_step(const gsgpu_ensemble *e) { return e ? e->kernels_per_step() : 0; }

int gsgpu_ensemble_num_particles(const gsgpu_ensemble *e) { return e ? e->P : 0; }

int gsgpu_ensemble_tuning(const gsgpu_ensemble *e, int *accel_threads, int *drift_threads)
{
    if (!e) return GRAV_POINTER_ERROR;
    if (accel_threads) *accel_threads = e->tuned ? e->tpb_accel : 0;
    if (drift_threads) *drift_threads = e->tuned ? e->tpb_drift : 0;
    return 0;
}

int gsgpu_ensemble_sort_tuning(const gsgpu_ensemble *e, int *pow2, int *threads, int n)
{
    if (!e || !pow2 || !threads) return GRAV_POINTER_ERROR;
    int k = 0;
    for (int c = 0; c < kSortClasses && k < n; ++c) {
        if (e->sort_first[c + 1] == e->sort_first[c]) continue;
        pow2[k] = e->sort_pow2[c];
        threads[k] = e->sort_tpb[c] > 0 ? e->sort_tpb[c]
                                        : std::min(1024, std::max(32, e->sort_pow2[c] / 2));
        ++k;
    }
    return k;
}

int gsgpu_ensemble_set_kernel_timing(gsgpu_ensemble *e, int enable)
{
    if (!e) return GRAV_POINTER_ERROR;
    e->timing = enable != 0;
    e->t_drift.enabled = e->t_accel.enabled = e->timing;
    e->t_drift.total_ms = e->t_accel.total_ms = 0.0;
    e->t_drift.launches = e->t_accel.launches = 0;
    return 0;
}

int gsgpu_ensemble_kernel_timing(const gsgpu_ensemble *e, double *drift_ms, double *accel_ms,
                                 int64_t *steps)
{
    if (!e) return GRAV_POINTER_ERROR;
    if (drift_ms) *drift_ms = e->t_drift.total_ms;
    if (accel_ms) *accel_ms = e->t_accel.total_ms;
    if (steps) *steps = e->t_accel.launches;
    return 0;
}

void gsgpu_ensemble_destroy(gsgpu_ensemble *e) { delete e; }

}  // extern "C"

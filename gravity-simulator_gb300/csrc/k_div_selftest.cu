// k_div_selftest.cu -- checks div_rcp (gs_div.cuh) against __ddiv_rn bit for
// bit on the GPU: random operand pairs over the whole finite double range,
// and the Stumpff series' fixed divisors over the range the series sees
// (|z| <= 0.1) and over the whole range.  A test entry point; nothing else
// calls it.
#include "gs_div.cuh"
#include "gs_internal.h"

namespace gs {

namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long z)
{
    // SplitMix64 finaliser (Steele, Lea and Flood, "Fast splittable
    // pseudorandom number generators", OOPSLA 2014)
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

__device__ __forceinline__ bool same_bits(double a, double b)
{
    return __double_as_longlong(a) == __double_as_longlong(b) || (a != a && b != b);
}

constexpr int kDivisors = 13;
__constant__ double c_div[kDivisors] = {210.0, 156.0, 110.0, 72.0, 42.0, 20.0, 6.0,
                                         182.0, 132.0, 90.0, 56.0, 30.0, 12.0};

__global__ void k_div_selftest(long long n, unsigned long long seed,
                               unsigned long long *mismatch)
{
    unsigned long long bad = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long r0 = mix64(seed ^ (2 * i)), r1 = mix64(seed ^ (2 * i + 1));
        // any bit pattern: every exponent, subnormals, zeros, infinities, NaNs
        const double a = __longlong_as_double((long long)r0);
        const double b = __longlong_as_double((long long)r1);
        bad += !same_bits(div_rcp(a, b, __drcp_rn(b)), __ddiv_rn(a, b));
        // the fixed divisors: z in [-0.1, 0.1] and z of any pattern
        const double zs = 0.2 * ((double)(r1 >> 11) * 0x1p-53) - 0.1;
        const int k = (int)(r0 % kDivisors);
        const double c = c_div[k], rc = 1.0 / c;
        bad += !same_bits(div_rcp(zs, c, rc), __ddiv_rn(zs, c));
        bad += !same_bits(div_rcp(a, c, rc), __ddiv_rn(a, c));
    }
    for (int o = 16; o > 0; o >>= 1) bad += __shfl_down_sync(0xffffffffu, bad, o);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(mismatch, bad);
}

}  // namespace

}  // namespace gs

// Test entry point (no counterpart in the reference): 3 n quotients formed
// by div_rcp and by __ddiv_rn from seeded random operands; *mismatches
// receives how many differ in any bit.
extern "C" int gsgpu_fp64_division_selftest(long long n, unsigned long long seed,
                                            long long *mismatches)
{
    using namespace gs;
    if (!mismatches) return GRAV_POINTER_ERROR;
    if (n < 1) return GRAV_VALUE_ERROR;
    const DeviceInfo *dev = nullptr;
    ErrorStatus st = device_info(&dev);
    if (st.return_code == GRAV_SUCCESS) {
        DBuf d;
        st = d.reserve(sizeof(unsigned long long));
        if (st.return_code == GRAV_SUCCESS) {
            cudaError_t e = cudaMemset(d.p, 0, sizeof(unsigned long long));
            if (e == cudaSuccess) {
                k_div_selftest<<<dev->sm_count * 8, 256>>>(n, seed, d.as<unsigned long long>());
                e = cudaGetLastError();
            }
            unsigned long long h = 0;
            if (e == cudaSuccess) e = cudaMemcpy(&h, d.p, sizeof(h), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess)
                st = GS_RAISE(GRAV_FAILURE, "division selftest: %s", cudaGetErrorString(e));
            *mismatches = (long long)h;
        }
    }
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    return GRAV_SUCCESS;
}

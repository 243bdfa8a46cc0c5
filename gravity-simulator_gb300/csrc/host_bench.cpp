// host_bench.cpp -- grav_sim's acceleration benchmark and the helpers its
// example program links against: benchmark_acceleration
// (src/acceleration.c:369-506), get_initialized_system (src/system.c:38-66),
// init_pcg_rng / grav_randrange / grav_get_current_time (src/utils.c:20-82)
// and the error helpers behind the WRAP_* macros of src/error.h.
//
// benchmark_acceleration keeps the reference's contract: it runs each
// acceleration parameter set num_times[i] times through acceleration(),
// times every call with CLOCK_MONOTONIC, keeps the first call of set 0 as the
// reference accelerations, and reports per set the mean and sample standard
// deviation of the run times and the mean absolute error of the set's first
// call against the reference, summed over the three components and divided
// by the particle count.  The GPU method codes are the ones it accepts (the
// library has no CPU path).  Unlike the reference, the reference
// accelerations start at zero, so an MAE printed while set 0 is skipped
// compares with zero rather than with uninitialised memory.
#include "gs_internal.h"

#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <vector>

namespace {

// Mean and standard deviation with ddof = 1 of n run times
// (src/math_functions.c:78-121).
double mean_of(const std::vector<double> &v)
{
    double s = 0.0;
    for (double t : v) s += t;
    return s / (double)v.size();
}

double std_of(const std::vector<double> &v)
{
    if (v.size() <= 1) return 0.0;
    const double mu = mean_of(v);
    double s = 0.0;
    for (double t : v) s += (t - mu) * (t - mu);
    return std::sqrt(s / ((double)v.size() - 1.0));
}

const char *method_name(int method)
{
    switch (method) {
    case GRAV_GPU_PAIRWISE: return "Pairwise (GPU, compensated FP32)";
    case GRAV_GPU_MASSLESS: return "Massless (GPU)";
    case GRAV_GPU_BARNES_HUT: return "Barnes-Hut (GPU)";
    case GRAV_GPU_BH_LEARNED: return "Barnes-Hut + learned residual (GPU)";
    case GRAV_GPU_BARNES_HUT_QUAD: return "Barnes-Hut, quadrupole cells (GPU)";
    case GRAV_GPU_BARNES_HUT_GROUP: return "Barnes-Hut group walk (GPU)";
    case GRAV_GPU_BARNES_HUT_GROUP_MONO: return "Barnes-Hut group walk, monopole cells (GPU)";
    case GRAV_GPU_PAIRWISE_FP64: return "Pairwise (GPU, FP64 reference order)";
    case GRAV_GPU_BARNES_HUT_COMPAT: return "Barnes-Hut, reference tree (GPU)";
    default: return nullptr;
    }
}

// PCG32 (O'Neill, "PCG: A Family of Simple Fast Space-Efficient
// Statistically Good Algorithms for Random Number Generation", 2014): a
// 64-bit LCG state advanced by the multiplier 6364136223846793005 and the
// stream increment, output by the xorshift-high / random-rotation
// permutation (XSH RR) of the old state.
uint32_t pcg32_next(pcg32_random_t *r)
{
    const uint64_t old = r->state;
    r->state = old * 6364136223846793005ULL + r->inc;
    const uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
}

void pcg32_seed(pcg32_random_t *r, uint64_t initstate, uint64_t initseq)
{
    r->state = 0u;
    r->inc = (initseq << 1u) | 1u;
    (void)pcg32_next(r);
    r->state += initstate;
    (void)pcg32_next(r);
}

}  // namespace

extern "C" {

// src/utils.c:20-25
double grav_get_current_time(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + (double)ts.tv_nsec / 1.0e9;
}

// src/utils.c:61-67: seeded from the clock, the stream from the address of
// the generator.
pcg32_random_t init_pcg_rng(void)
{
    pcg32_random_t rng;
    pcg32_seed(&rng, (uint64_t)time(nullptr), (uint64_t)(intptr_t)&rng);
    return rng;
}

// src/utils.c:69-82: min + (max - min) u with u = r / 2^32 in [0, 1).
double grav_randrange(const double min, const double max, pcg32_random_t *rng)
{
    const double u = std::ldexp((double)pcg32_next(rng), -32);
    return min + (max - min) * u;
}

// src/system.c:38-66
ErrorStatus get_initialized_system(System *system, const int num_particles)
{
    if (!system) return GS_RAISE(GRAV_POINTER_ERROR, "System is NULL");
    *system = get_new_system();
    system->num_particles = num_particles;
    const size_t n = num_particles > 0 ? (size_t)num_particles : 0;
    system->particle_ids = static_cast<int *>(std::malloc(n * sizeof(int)));
    system->x = static_cast<double *>(std::calloc(n * 3, sizeof(double)));
    system->v = static_cast<double *>(std::calloc(n * 3, sizeof(double)));
    system->m = static_cast<double *>(std::calloc(n, sizeof(double)));
    if (!system->particle_ids || !system->x || !system->v || !system->m) {
        free_system(system);
        return GS_RAISE(GRAV_MEMORY_ERROR, "Failed to allocate memory for system");
    }
    for (int i = 0; i < num_particles; ++i) system->particle_ids[i] = i;
    return gs::ok();
}

// The error helpers of src/error.h's WRAP_RAISE_ERROR / WRAP_RAISE_ERROR_FMT /
// WRAP_TRACEBACK / WRAP_RAISE_WARNING macros (src/error.c:35-455), for
// programs written against grav_sim's headers.
ErrorStatus raise_error(const char *error_file, const int error_line, const char *error_func,
                        const int error_code, const char *error_msg)
{
    return gs::raise_error(error_code, error_file, error_line, error_func, "%s", error_msg);
}

ErrorStatus raise_error_fmt(const char *error_file, const int error_line, const char *error_func,
                            const int error_code, const char *format, ...)
{
    char msg[1024];
    va_list ap;
    va_start(ap, format);
    std::vsnprintf(msg, sizeof(msg), format, ap);
    va_end(ap);
    return gs::raise_error(error_code, error_file, error_line, error_func, "%s", msg);
}

void raise_warning(const char *warning_file, const int warning_line, const char *warning_func,
                   const char *warning_msg)
{
    std::fprintf(stderr, "Warning: In \"%s\", line %d in %s:\n    %s\n", warning_file,
                 warning_line, warning_func, warning_msg);
}

ErrorStatus raise_warning_fmt(const char *warning_file, const int warning_line,
                              const char *warning_func, const char *format, ...)
{
    char msg[1024];
    va_list ap;
    va_start(ap, format);
    const int len = std::vsnprintf(msg, sizeof(msg), format, ap);
    va_end(ap);
    if (len < 0) return GS_RAISE(GRAV_UNKNOWN_ERROR, "Failed to encode warning message");
    if (len >= (int)sizeof(msg)) return GS_RAISE(GRAV_UNKNOWN_ERROR, "Warning message is truncated");
    raise_warning(warning_file, warning_line, warning_func, msg);
    return gs::ok();
}

ErrorStatus traceback(ErrorStatus error_status, const char *function_call_source_code,
                      const char *error_file, const int error_line, const char *error_func)
{
    if (error_status.return_code == GRAV_SUCCESS) return error_status;
    return gs::traceback(error_status, function_call_source_code, error_file, error_line,
                         error_func);
}

// src/acceleration.c:369-506
ErrorStatus benchmark_acceleration(const System *system,
                                   const AccelerationParam *acceleration_params,
                                   const int num_acceleration_params,
                                   const int *num_times_acceleration_param)
{
    if (!system || !acceleration_params || !num_times_acceleration_param)
        return GS_RAISE(GRAV_POINTER_ERROR, "benchmark_acceleration: NULL argument");
    const int n = system->num_particles;
    if (n <= 0)
        return GS_RAISE(GRAV_VALUE_ERROR, "Number of particles must be positive. Got: %d", n);
    std::vector<double> reference_a, a;
    try {
        reference_a.assign((size_t)n * 3, 0.0);
        a.assign((size_t)n * 3, 0.0);
    } catch (...) {
        return GS_RAISE(GRAV_MEMORY_ERROR, "Failed to allocate memory for acceleration arrays");
    }

    std::fputs("Benchmarking acceleration...\n", stdout);
    for (int i = 0; i < num_acceleration_params; ++i) {
        const AccelerationParam *param = &acceleration_params[i];
        const int num_times = num_times_acceleration_param[i];
        if (num_times <= 0) {
            std::printf("Test %d:    Skipped since num_times: %d <= 0\n\n", i, num_times);
            continue;
        }
        std::vector<double> run_time((size_t)num_times, 0.0);
        double mae = 0.0;
        for (int j = 0; j < num_times; ++j) {
            double *out = (i == 0 && j == 0) ? reference_a.data() : a.data();
            const double t0 = grav_get_current_time();
            ErrorStatus st = acceleration(out, system, param);
            if (st.return_code != GRAV_SUCCESS)
                return gs::traceback(st, "acceleration(a, system, acceleration_param)", __FILE__,
                                     __LINE__, __func__);
            run_time[(size_t)j] += grav_get_current_time() - t0;
            if (i != 0 && j == 0) {
                for (int k = 0; k < n; ++k)
                    mae += std::fabs(reference_a[3 * (size_t)k + 0] - a[3 * (size_t)k + 0]) +
                           std::fabs(reference_a[3 * (size_t)k + 1] - a[3 * (size_t)k + 1]) +
                           std::fabs(reference_a[3 * (size_t)k + 2] - a[3 * (size_t)k + 2]);
                mae /= n;
            }
        }
        std::printf("Test %d:", i);
        const char *name = method_name(param->method);
        if (!name)
            return GS_RAISE(GRAV_VALUE_ERROR, "Unknown acceleration method. Got: %d", param->method);
        std::printf("    Method: %s\n", name);
        std::printf("    Number of times: %d\n", num_times);
        std::printf("    Avg time: %.3g (+- %.3g) s\n", mean_of(run_time), std_of(run_time));
        std::printf("    MAE: %.3g\n", mae);
        std::printf("\n");
    }
    std::fflush(stdout);
    return gs::ok();
}

}  // extern "C"

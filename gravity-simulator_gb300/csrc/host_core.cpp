// host_core.cpp -- errors, device buffers, timers, engine factory and the
// small parameter helpers of grav_sim's C ABI.
#include "gs_internal.h"

#include <cufft.h>

#include <atomic>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

namespace gs {

// ---- errors (same ErrorStatus contract as src/error.c) ------------------
ErrorStatus ok()
{
    ErrorStatus st;
    st.return_code = GRAV_SUCCESS;
    st.traceback = nullptr;
    st.traceback_code_ = -1;
    return st;
}

static const char *code_name(int code)
{
    switch (code) {
    case GRAV_VALUE_ERROR: return "ValueError";
    case GRAV_POINTER_ERROR: return "PointerError";
    case GRAV_MEMORY_ERROR: return "MemoryError";
    case GRAV_OS_ERROR: return "OSError";
    case GRAV_NOT_IMPLEMENTED_ERROR: return "NotImplementedError";
    case GRAV_FAILURE: return "Failure";
    default: return "UnknownError";
    }
}

static char *dup_string(const std::string &s)
{
    char *p = static_cast<char *>(std::malloc(s.size() + 1));
    if (p) std::memcpy(p, s.c_str(), s.size() + 1);
    return p;
}

ErrorStatus raise_error(int code, const char *file, int line, const char *func, const char *fmt,
                        ...)
{
    char msg[1024];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(msg, sizeof(msg), fmt, ap);
    va_end(ap);
    std::string tb;
    tb += "    File \"";
    tb += file;
    tb += "\", line " + std::to_string(line) + " in " + func + "\n";
    tb += std::string(code_name(code)) + ": " + msg + "\n";
    ErrorStatus st;
    st.return_code = code;
    st.traceback = dup_string(tb);
    st.traceback_code_ = st.traceback ? 0 : 1;
    return st;
}

ErrorStatus traceback(ErrorStatus st, const char *call, const char *file, int line,
                      const char *func)
{
    std::string tb;
    tb += "    File \"";
    tb += file;
    tb += "\", line " + std::to_string(line) + " in " + func + "\n        " + call + "\n";
    if (st.traceback) tb += st.traceback;
    std::free(st.traceback);
    st.traceback = dup_string(tb);
    st.traceback_code_ = st.traceback ? 0 : 1;
    return st;
}

ErrorStatus cuda_error(cudaError_t e, const char *what, const char *file, int line,
                       const char *func)
{
    const int code = (e == cudaErrorMemoryAllocation) ? GRAV_MEMORY_ERROR : GRAV_FAILURE;
    return raise_error(code, file, line, func, "CUDA error %s (%s) in %s", cudaGetErrorName(e),
                       cudaGetErrorString(e), what);
}

// ---- device buffers -----------------------------------------------------
DBuf::~DBuf() { release(); }

void DBuf::release()
{
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

// Host-side fault injection for tests: when set to k > 0, the k-th device
// allocation from now on fails as an out-of-memory cudaMalloc would.
static std::atomic<int> g_fail_alloc_in{0};

ErrorStatus DBuf::reserve(size_t b)
{
    if (b <= bytes && p) return ok();
    release();
    if (b == 0) b = 16;
    int k = g_fail_alloc_in.load();
    while (k > 0 && !g_fail_alloc_in.compare_exchange_weak(k, k - 1)) {
    }
    cudaError_t e = (k == 1) ? cudaErrorMemoryAllocation : cudaMalloc(&p, b);
    if (e != cudaSuccess) {
        p = nullptr;
        (void)cudaGetLastError();
        return GS_RAISE(e == cudaErrorMemoryAllocation ? GRAV_MEMORY_ERROR : GRAV_FAILURE,
                        "cudaMalloc of %zu bytes failed: %s", b, cudaGetErrorString(e));
    }
    bytes = b;
    return ok();
}

// ---- device -------------------------------------------------------------
ErrorStatus device_info(const DeviceInfo **out)
{
    static std::mutex mu;
    static DeviceInfo info[kMaxDevices];
    static bool done[kMaxDevices] = {};
    std::lock_guard<std::mutex> lock(mu);
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count < 1) {
        (void)cudaGetLastError();
        return GS_RAISE(GRAV_FAILURE, "no CUDA device available (%s)", cudaGetErrorString(e));
    }
    int dev = 0;
    GS_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return GS_RAISE(GRAV_FAILURE, "device ordinal %d is beyond the %d this library tracks", dev,
                        kMaxDevices);
    if (!done[dev]) {
        DeviceInfo &d = info[dev];
        d.id = dev;
        cudaDeviceProp prop;
        GS_CUDA(cudaGetDeviceProperties(&prop, dev));
        d.sm_count = prop.multiProcessorCount;
        d.cc_major = prop.major;
        d.cc_minor = prop.minor;
        std::snprintf(d.name, sizeof(d.name), "%s", prop.name);
        if (prop.major < 10)
            return GS_RAISE(GRAV_FAILURE, "device %s (sm_%d%d) is not a Blackwell GPU; this "
                            "library is built for sm_103a only", prop.name, prop.major, prop.minor);
        done[dev] = true;
    }
    *out = &info[dev];
    return ok();
}

// ---- force timer --------------------------------------------------------
ErrorStatus ForceTimer::begin(cudaStream_t s)
{
    if (!enabled) return ok();
    if (used + 2 > ev.size()) {
        for (int k = 0; k < 64; ++k) {
            cudaEvent_t e;
            GS_CUDA(cudaEventCreate(&e));
            ev.push_back(e);
        }
    }
    GS_CUDA(cudaEventRecord(ev[used], s));
    return ok();
}

ErrorStatus ForceTimer::end(cudaStream_t s)
{
    if (!enabled) return ok();
    GS_CUDA(cudaEventRecord(ev[used + 1], s));
    used += 2;
    return ok();
}

ErrorStatus ForceTimer::collect()
{
    for (size_t k = 0; k + 1 < used; k += 2) {
        float ms = 0.0f;
        GS_CUDA(cudaEventSynchronize(ev[k + 1]));
        GS_CUDA(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
        total_ms += ms;
        ++launches;
    }
    used = 0;
    return ok();
}

ForceTimer::~ForceTimer()
{
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
}

// ---- engines --------------------------------------------------------------
bool is_gpu_method(int method)
{
    switch (method) {
    case GRAV_GPU_PAIRWISE:
    case GRAV_GPU_PAIRWISE_FP64:
    case GRAV_GPU_MASSLESS:
    case GRAV_GPU_BARNES_HUT:
    case GRAV_GPU_BARNES_HUT_COMPAT:
    case GRAV_GPU_BARNES_HUT_QUAD:
    case GRAV_GPU_BARNES_HUT_GROUP:
    case GRAV_GPU_BARNES_HUT_GROUP_MONO:
    case GRAV_GPU_BH_LEARNED:
        return true;
    default:
        return false;
    }
}

ErrorStatus make_engine(int method, std::unique_ptr<Engine> &out)
{
    switch (method) {
    case GRAV_GPU_PAIRWISE: out = make_direct_engine(false); break;
    case GRAV_GPU_PAIRWISE_FP64: out = make_direct_engine(true); break;
    case GRAV_GPU_MASSLESS: out = make_massless_engine(); break;
    case GRAV_GPU_BARNES_HUT: out = make_barnes_hut_engine(false); break;
    case GRAV_GPU_BARNES_HUT_COMPAT: out = make_barnes_hut_engine(true); break;
    case GRAV_GPU_BARNES_HUT_QUAD: out = make_barnes_hut_engine(false, true); break;
    case GRAV_GPU_BARNES_HUT_GROUP: out = make_barnes_hut_engine(false, true, true); break;
    case GRAV_GPU_BARNES_HUT_GROUP_MONO: out = make_barnes_hut_engine(false, false, true); break;
    case GRAV_GPU_BH_LEARNED: out = make_learned_engine(); break;
    default:
        return GS_RAISE(GRAV_VALUE_ERROR,
                        "Unknown acceleration method. Got: %d (this library computes on the GPU "
                        "only: use 101 pairwise, 102 massless, 103 Barnes-Hut, 104 learned "
                        "Barnes-Hut, 105 quadrupole Barnes-Hut, 106 / 107 group Barnes-Hut, 111 "
                        "FP64 "
                        "pairwise, 113 "
                        "reference-compatible Barnes-Hut)",
                        method);
    }
    if (!out) return GS_RAISE(GRAV_NOT_IMPLEMENTED_ERROR, "acceleration method %d is not built",
                              method);
    return ok();
}

}  // namespace gs

// ---- C ABI: errors and parameter helpers ----------------------------------
using namespace gs;

extern "C" {

ErrorStatus make_success_error_status(void) { return ok(); }

// Test hook (no reference counterpart): the k-th device allocation from now
// on fails with an out-of-memory error; k = 0 switches the injection off.
void gsgpu_test_fail_allocation(int k)
{
    g_fail_alloc_in.store(k > 0 ? k : 0);
}

void free_traceback(ErrorStatus *error_status)
{
    if (!error_status) return;
    std::free(error_status->traceback);
    error_status->traceback = nullptr;
}

void print_and_free_traceback(ErrorStatus *error_status)
{
    if (!error_status) return;
    std::fprintf(stderr, "Traceback (most recent call last):\n%s",
                 error_status->traceback ? error_status->traceback : "    (no traceback)\n");
    free_traceback(error_status);
}

// src/system.c:26-36: G defaults to its value in AU^3 day^-2 Msun^-1.
System get_new_system(void)
{
    System s;
    s.num_particles = 0;
    s.particle_ids = nullptr;
    s.x = nullptr;
    s.v = nullptr;
    s.m = nullptr;
    s.G = 0.000295912208284119496676630;
    return s;
}

// src/acceleration.c:62-71
AccelerationParam get_new_acceleration_param(void)
{
    AccelerationParam p;
    p.method = GRAV_GPU_PAIRWISE;
    p.opening_angle = 1.0;
    p.softening_length = 0.0;
    p.max_num_particles_per_leaf = -1;
    return p;
}

// src/acceleration.c:73-129 with the GPU method codes.
ErrorStatus finalize_acceleration_param(AccelerationParam *p)
{
    if (!p) return GS_RAISE(GRAV_POINTER_ERROR, "Acceleration parameter pointer is NULL");
    if (!is_gpu_method(p->method))
        return GS_RAISE(GRAV_VALUE_ERROR, "Unknown acceleration method. Got: %d", p->method);
    if (p->softening_length < 0.0)
        return GS_RAISE(GRAV_VALUE_ERROR, "Softening length is negative. Got: %.3g",
                        p->softening_length);
    const bool bh = p->method == GRAV_GPU_BARNES_HUT || p->method == GRAV_GPU_BARNES_HUT_COMPAT ||
                    p->method == GRAV_GPU_BARNES_HUT_QUAD || p->method == GRAV_GPU_BH_LEARNED ||
                    p->method == GRAV_GPU_BARNES_HUT_GROUP ||
                    p->method == GRAV_GPU_BARNES_HUT_GROUP_MONO;
    if (bh && p->opening_angle < 0.0)
        return GS_RAISE(GRAV_VALUE_ERROR, "Opening angle is negative. Got: %.3g",
                        p->opening_angle);
    if (bh) {
        // The reference's default is one particle per leaf.  The group walks
        // (106, 107, and the walks of the learned method 104) evaluate opened
        // leaves as particle lists, and leaves of up to 16 particles make them
        // faster at the same accuracy (a smaller tree to build and to
        // traverse; 16 was the fastest of 4, 8, 12, 16, 24 and 32 on the
        // galaxy pair at N = 1,048,576 and 2,097,152), so that is their
        // default.
        const bool group = p->method == GRAV_GPU_BARNES_HUT_GROUP ||
                           p->method == GRAV_GPU_BARNES_HUT_GROUP_MONO ||
                           p->method == GRAV_GPU_BH_LEARNED;
        if (p->max_num_particles_per_leaf == -1)
            p->max_num_particles_per_leaf = group ? 16 : 1;
        else if (p->max_num_particles_per_leaf < 1)
            return GS_RAISE(GRAV_VALUE_ERROR,
                            "Maximum number of particles per leaf must be positive. Got: %d",
                            p->max_num_particles_per_leaf);
    }
    return ok();
}

// src/integrator.c:119-129
IntegratorParam get_new_integrator_param(void)
{
    IntegratorParam p;
    p.integrator = -1;
    p.dt = -1.0;
    p.tolerance = -1.0;
    p.initial_dt = -1.0;
    p.whfast_remove_invalid_particles = true;
    return p;
}

// src/output.c:85-98
OutputParam get_new_output_param(void)
{
    OutputParam p;
    p.method = OUTPUT_METHOD_DISABLED;
    p.output_dir = nullptr;
    p.output_initial = false;
    p.output_interval = -1.0;
    p.coordinate_output_dtype = 2;
    p.velocity_output_dtype = 2;
    p.mass_output_dtype = 2;
    p.output_count_ = 0;
    return p;
}

Settings get_new_settings(void)
{
    static bool never_exit = false;
    Settings s;
    s.verbose = 2;
    s.enable_progress_bar = false;
    s.is_exit_ptr = &never_exit;
    return s;
}

int gsgpu_device_info(char *name, int len, int *sm_count, int *cc_major, int *cc_minor)
{
    const DeviceInfo *d = nullptr;
    ErrorStatus st = device_info(&d);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    if (name && len > 0) std::snprintf(name, (size_t)len, "%s", d->name);
    if (sm_count) *sm_count = d->sm_count;
    if (cc_major) *cc_major = d->cc_major;
    if (cc_minor) *cc_minor = d->cc_minor;
    return 0;
}

// src/grav_sim.h:92 (src/grav_sim.c:630-700): what the library was built
// with, in the reference's section layout (grav_sim's `python -m grav_sim`
// and launch_simulation at normal verbosity print it).  This library's
// facts: the device architecture, the CUDA runtime and cuFFT it was built
// against, its own HDF5 snapshot writer.
void print_compilation_info(void)
{
    const char *line = "-----------------------------------------------------------------\n";
    std::fputs(line, stdout);
    std::fputs("grav_sim force-evaluation path for GB300 (sm_103a)\n\n", stdout);
#ifdef __linux__
    std::fputs("Operating System: Linux\n", stdout);
#else
    std::fputs("Operating System: Unknown\n", stdout);
#endif
    std::fputs("Compilation Info:\n", stdout);
    std::printf("  CUDA runtime: %d.%d\n", CUDART_VERSION / 1000, (CUDART_VERSION % 1000) / 10);
    std::fputs("  Device code: sm_103a (no CPU fallback)\n", stdout);
    std::fputs("  Compiled with OpenMP: false\n", stdout);
    std::fputs("  HDF5 snapshots: true (written and read without libhdf5)\n", stdout);
    int fft_version = 0;
    if (cufftGetVersion(&fft_version) == CUFFT_SUCCESS)
        std::printf("  Particle-mesh transforms: cuFFT %d\n", fft_version);
    else
        std::fputs("  Particle-mesh transforms: cuFFT\n", stdout);
    std::fputs("\n", stdout);
    std::printf("Build time: %s %s\n", __DATE__, __TIME__);
#if defined(__GNUC__) && !defined(__clang__)
    std::printf("Compiler: GCC (version: %d)\n", __GNUC__);
#endif
    std::fputs(line, stdout);
    std::fflush(stdout);   // before any output of the caller's own runtime
}

void free_memory_int32(int32_t *ptr) { std::free(ptr); }
void free_memory_double(double *ptr) { std::free(ptr); }

int32_t load_built_in_system_python(const char *system_name, int *num_particles_ptr,
                                    int32_t **particle_ids_ptr, double **x_ptr, double **v_ptr,
                                    double **m_ptr, double *G_ptr)
{
    (void)num_particles_ptr; (void)particle_ids_ptr; (void)x_ptr; (void)v_ptr; (void)m_ptr;
    (void)G_ptr;
    ErrorStatus st = GS_RAISE(GRAV_NOT_IMPLEMENTED_ERROR,
                              "built-in system \"%s\": initial conditions are not part of the "
                              "GPU library", system_name ? system_name : "(null)");
    print_and_free_traceback(&st);
    return GRAV_NOT_IMPLEMENTED_ERROR;
}

// Keplerian elements -> Cartesian for a two-body orbit with total mass M
// (same element convention as src/utils.c:82-141: a, e, i, argument of
// periapsis, longitude of ascending node, true anomaly).
void keplerian_to_cartesian_python(double *x, double *y, double *z, double *v_x, double *v_y,
                                   double *v_z, double a, double e, double inc, double argp,
                                   double node, double f, double total_mass, double G)
{
    const double mu = G * total_mass;
    const double p = a * (1.0 - e * e);
    const double r = p / (1.0 + e * std::cos(f));
    const double xo = r * std::cos(f), yo = r * std::sin(f);
    const double h = std::sqrt(mu * p);
    const double vxo = -mu / h * std::sin(f), vyo = mu / h * (e + std::cos(f));
    const double cO = std::cos(node), sO = std::sin(node);
    const double cw = std::cos(argp), sw = std::sin(argp);
    const double ci = std::cos(inc), si = std::sin(inc);
    const double r11 = cO * cw - sO * sw * ci, r12 = -cO * sw - sO * cw * ci;
    const double r21 = sO * cw + cO * sw * ci, r22 = -sO * sw + cO * cw * ci;
    const double r31 = sw * si, r32 = cw * si;
    *x = r11 * xo + r12 * yo;
    *y = r21 * xo + r22 * yo;
    *z = r31 * xo + r32 * yo;
    *v_x = r11 * vxo + r12 * vyo;
    *v_y = r21 * vxo + r22 * vyo;
    *v_z = r31 * vxo + r32 * vyo;
}

bool linear_octree_check_if_included(int64_t morton_index_i, int64_t morton_index_j, int level)
{
    const int sh = 3 * (MORTON_MAX_LEVEL - level);
    return (morton_index_i >> sh) == (morton_index_j >> sh);
}

}  // extern "C"

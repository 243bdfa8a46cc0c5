// host_output.cpp -- CSV and HDF5 snapshots written by launch_simulation.
//
// The output parameters are checked as src/output.c:100-239 checks them
// (method, positive interval, a directory path ending in '/', or
// snapshots_YYYYMMDD_HHMMSS/ when none is given, created if missing), and a
// snapshot is the reference's CSV file (src/output.c:380-470): the path
// "<dir>snapshot_%05d.csv" numbered by OutputParam.output_count_, four
// metadata lines, the header line, then one line per particle with "%.17g"
// (double) or "%.8g" (float output dtype) fields.  An HDF5 snapshot
// (src/output.c:483-695) is "<dir>snapshot_%05d.hdf5", written by
// write_snapshot_hdf5 (host_hdf5.cpp).
//
// Snapshots inside the step loop are asynchronous: the state is copied
// device->host on the run's stream into one of two pinned slots, an event
// marks the copy, and a writer thread waits for the event and formats the
// file while the GPU runs the next steps.  The loop waits only when both
// slots are still being written.
#include "gs_internal.h"

#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <deque>
#include <mutex>
#include <string>
#include <sys/stat.h>
#include <sys/types.h>
#include <thread>

namespace gs {

ErrorStatus output_prepare(OutputParam *op, const Settings *settings)
{
    if (!op) return GS_RAISE(GRAV_POINTER_ERROR, "output_param is NULL");
    switch (op->method) {
    case OUTPUT_METHOD_DISABLED:
        return ok();
    case OUTPUT_METHOD_CSV:
    case OUTPUT_METHOD_HDF5:
        break;
    default:
        return GS_RAISE(GRAV_VALUE_ERROR, "Unknown output method. Got: %d", op->method);
    }
    if (op->output_interval <= 0.0)
        return GS_RAISE(GRAV_VALUE_ERROR, "Output interval must be positive. Got: %.17g",
                        op->output_interval);
    if (!op->output_dir) {
        // snapshots_YYYYMMDD_HHMMSS/ (the library keeps the string)
        static thread_local char name[64];
        const std::time_t now = std::time(nullptr);
        std::strftime(name, sizeof(name), "snapshots_%Y%m%d_%H%M%S/", std::localtime(&now));
        op->output_dir = name;
    } else {
        const size_t len = std::strlen(op->output_dir);
        if (len == 0 || op->output_dir[len - 1] != '/')
            return GS_RAISE(GRAV_VALUE_ERROR,
                            "Directory path for storing snapshots must end with a trailing slash "
                            "(\"/\"). Got: \"%s\".",
                            op->output_dir);
    }
    if (mkdir(op->output_dir, 0777) == -1) {
        struct stat st;
        if (stat(op->output_dir, &st) != 0)
            return GS_RAISE(GRAV_OS_ERROR, "Failed to access path for storing snapshots: \"%s\".",
                            op->output_dir);
        if ((st.st_mode & S_IFDIR) && settings && settings->verbose >= 1)
            std::fprintf(stderr,
                         "Warning: Directory for storing snapshots already exists. The files will "
                         "be overwritten. Directory: \"%s\".\n",
                         op->output_dir);
    }
    return ok();
}

namespace {

// src/output.c:340-470, file number given.
ErrorStatus write_csv(const OutputParam *op, int index, int n, const int *ids, const double *x,
                      const double *v, const double *m, double G, double t, double dt)
{
    char path[4096];
    const int len = std::snprintf(path, sizeof(path), "%ssnapshot_%05d.csv", op->output_dir, index);
    if (len < 0) return GS_RAISE(GRAV_VALUE_ERROR, "Failed to get storing file path string");
    if (len >= (int)sizeof(path)) return GS_RAISE(GRAV_VALUE_ERROR, "Storing file path string is truncated.");
    std::FILE *f = std::fopen(path, "w");
    if (!f)
        return GS_RAISE(GRAV_OS_ERROR, "Failed to open file for storing snapshots: \"%s\".", path);
    std::fprintf(f, "# num_particles: %d\n", n);
    std::fprintf(f, "# G: %.17g\n", G);
    std::fprintf(f, "# time: %.17g\n", t);
    std::fprintf(f, "# dt: %.17g\n", dt);
    std::fputs("particle_id,m,x,y,z,vx,vy,vz\n", f);
    const char *fm = op->mass_output_dtype == OUTPUT_DTYPE_FLOAT ? "%.8g," : "%.17g,";
    const char *fx = op->coordinate_output_dtype == OUTPUT_DTYPE_FLOAT ? "%.8g," : "%.17g,";
    const bool vf = op->velocity_output_dtype == OUTPUT_DTYPE_FLOAT;
    const char *fv = vf ? "%.8g," : "%.17g,";
    const char *fv_last = vf ? "%.8g\n" : "%.17g\n";
    for (int i = 0; i < n; ++i) {
        std::fprintf(f, "%d,", ids[i]);
        std::fprintf(f, fm, m[i]);
        std::fprintf(f, fx, x[3 * i]);
        std::fprintf(f, fx, x[3 * i + 1]);
        std::fprintf(f, fx, x[3 * i + 2]);
        std::fprintf(f, fv, v[3 * i]);
        std::fprintf(f, fv, v[3 * i + 1]);
        std::fprintf(f, fv_last, v[3 * i + 2]);
    }
    const bool bad = std::ferror(f) != 0;
    std::fclose(f);
    if (bad) return GS_RAISE(GRAV_OS_ERROR, "Failed to write snapshot file: \"%s\".", path);
    return ok();
}

// src/output.c:241-290: the snapshot in the file format the method names.
ErrorStatus write_snapshot(const OutputParam *op, int index, int n, const int *ids,
                           const double *x, const double *v, const double *m, double G, double t,
                           double dt)
{
    if (op->method != OUTPUT_METHOD_HDF5) return write_csv(op, index, n, ids, x, v, m, G, t, dt);
    char path[4096];
    const int len = std::snprintf(path, sizeof(path), "%ssnapshot_%05d.hdf5", op->output_dir, index);
    if (len < 0) return GS_RAISE(GRAV_VALUE_ERROR, "Failed to get storing file path string");
    if (len >= (int)sizeof(path)) return GS_RAISE(GRAV_VALUE_ERROR, "Storing file path string is truncated.");
    return write_snapshot_hdf5(path, n, ids, x, v, m, t,
                               op->coordinate_output_dtype == OUTPUT_DTYPE_FLOAT,
                               op->velocity_output_dtype == OUTPUT_DTYPE_FLOAT,
                               op->mass_output_dtype == OUTPUT_DTYPE_FLOAT, nullptr);
}

template <class T> ErrorStatus pinned(T *&p, size_t count)
{
    GS_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&p), count * sizeof(T), cudaHostAllocDefault));
    return ok();
}

}  // namespace

ErrorStatus output_snapshot(OutputParam *op, int n, const int *ids, const double *x,
                            const double *v, const double *m, double G, double t, double dt)
{
    GS_TRY(write_snapshot(op, op->output_count_, n, ids, x, v, m, G, t, dt));
    ++op->output_count_;
    return ok();
}

ErrorStatus output_snapshot_cosmology(OutputParam *op, const CosmologicalSystem *system, double t)
{
    switch (op->method) {
    case OUTPUT_METHOD_DISABLED:
        break;
    case OUTPUT_METHOD_CSV:
        return GS_RAISE(GRAV_VALUE_ERROR,
                        "CSV output method is not supported for cosmological simulation.");
    case OUTPUT_METHOD_HDF5: {
        char path[4096];
        const int len = std::snprintf(path, sizeof(path), "%ssnapshot_%05d.hdf5", op->output_dir,
                                      op->output_count_);
        if (len < 0) return GS_RAISE(GRAV_VALUE_ERROR, "Failed to get storing file path string");
        if (len >= (int)sizeof(path))
            return GS_RAISE(GRAV_VALUE_ERROR, "Storing file path string is truncated.");
        const CosmologyHeader h = {system->omega_m, system->omega_lambda, system->unit_length,
                                   system->unit_mass, system->unit_time};
        GS_TRY(write_snapshot_hdf5(path, system->num_particles, system->particle_ids, system->x,
                                   system->v, system->m, t,
                                   op->coordinate_output_dtype == OUTPUT_DTYPE_FLOAT,
                                   op->velocity_output_dtype == OUTPUT_DTYPE_FLOAT,
                                   op->mass_output_dtype == OUTPUT_DTYPE_FLOAT, &h));
        break;
    }
    default:
        return GS_RAISE(GRAV_VALUE_ERROR, "Unknown output method. Got: %d", op->method);
    }
    ++op->output_count_;
    return ok();
}

class SnapshotWriter {
  public:
    SnapshotWriter(const OutputParam *op, const System *system) : op_(op), system_(system)
    {
        thread_ = std::thread([this] { run(); });
    }

    ~SnapshotWriter()
    {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        thread_.join();
        for (Slot &s : slots_) {
            if (s.ready) cudaEventDestroy(s.ready);
            cudaFreeHost(s.x);
            cudaFreeHost(s.v);
            cudaFreeHost(s.m);
            cudaFreeHost(s.ids);
            cudaFreeHost(s.cnt);
        }
    }

    ErrorStatus take(int index, int n, const double *d_x, const double *d_v, const int *d_ids,
                     const double *d_m, const int *d_cnt, cudaStream_t st, double t, double dt)
    {
        int k = -1;
        {
            std::unique_lock<std::mutex> lk(mu_);
            cv_.wait(lk, [&] { return failed_ || !slots_[0].busy || !slots_[1].busy; });
            if (failed_) return failure();
            k = slots_[0].busy ? 1 : 0;
            slots_[k].busy = true;
        }
        Slot &s = slots_[k];
        ErrorStatus e = fill(s, n, d_x, d_v, d_ids, d_m, d_cnt, st);
        if (e.return_code != GRAV_SUCCESS) {
            std::lock_guard<std::mutex> lk(mu_);
            s.busy = false;
            return e;
        }
        s.index = index;
        s.n = n;
        s.t = t;
        s.dt = dt;
        {
            std::lock_guard<std::mutex> lk(mu_);
            queue_.push_back(k);
        }
        cv_.notify_all();
        return ok();
    }

    ErrorStatus finish()
    {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return queue_.empty() && !slots_[0].busy && !slots_[1].busy; });
        if (failed_) return failure();
        return ok();
    }

  private:
    struct Slot {
        double *x = nullptr, *v = nullptr, *m = nullptr;
        int *ids = nullptr, *cnt = nullptr;
        size_t cap = 0;
        bool dev_ids = false, dev_m = false, dev_cnt = false;
        cudaEvent_t ready = nullptr;
        int index = 0, n = 0;
        double t = 0.0, dt = 0.0;
        bool busy = false;
    };

    ErrorStatus fill(Slot &s, int n, const double *d_x, const double *d_v, const int *d_ids,
                     const double *d_m, const int *d_cnt, cudaStream_t st)
    {
        const size_t N = (size_t)n;
        if (s.cap < N) {
            cudaFreeHost(s.x);
            cudaFreeHost(s.v);
            cudaFreeHost(s.m);
            cudaFreeHost(s.ids);
            s.x = s.v = s.m = nullptr;
            s.ids = nullptr;
            s.cap = 0;
            GS_TRY(pinned(s.x, 3 * N));
            GS_TRY(pinned(s.v, 3 * N));
            GS_TRY(pinned(s.m, N));
            GS_TRY(pinned(s.ids, N));
            s.cap = N;
        }
        if (!s.cnt) GS_TRY(pinned(s.cnt, 1));
        if (!s.ready) GS_CUDA(cudaEventCreateWithFlags(&s.ready, cudaEventDisableTiming));
        GS_CUDA(cudaMemcpyAsync(s.x, d_x, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, st));
        GS_CUDA(cudaMemcpyAsync(s.v, d_v, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, st));
        s.dev_ids = d_ids != nullptr;
        s.dev_m = d_m != nullptr;
        s.dev_cnt = d_cnt != nullptr;
        if (s.dev_ids)
            GS_CUDA(cudaMemcpyAsync(s.ids, d_ids, N * sizeof(int), cudaMemcpyDeviceToHost, st));
        if (s.dev_m)
            GS_CUDA(cudaMemcpyAsync(s.m, d_m, N * sizeof(double), cudaMemcpyDeviceToHost, st));
        if (s.dev_cnt)
            GS_CUDA(cudaMemcpyAsync(s.cnt, d_cnt, sizeof(int), cudaMemcpyDeviceToHost, st));
        GS_CUDA(cudaEventRecord(s.ready, st));
        return ok();
    }

    void run()
    {
        for (;;) {
            int k = -1;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return stop_ || !queue_.empty(); });
                if (queue_.empty()) return;
                k = queue_.front();
                queue_.pop_front();
            }
            Slot &s = slots_[k];
            ErrorStatus e = ok();
            const cudaError_t ce = cudaEventSynchronize(s.ready);
            if (ce != cudaSuccess) {
                e = GS_RAISE(GRAV_FAILURE, "snapshot copy failed: %s", cudaGetErrorString(ce));
            } else {
                int n = s.n;
                if (s.dev_cnt) n = *s.cnt < n ? *s.cnt : n;
                e = write_snapshot(op_, s.index, n, s.dev_ids ? s.ids : system_->particle_ids,
                                   s.x, s.v, s.dev_m ? s.m : system_->m, system_->G, s.t, s.dt);
            }
            std::lock_guard<std::mutex> lk(mu_);
            if (e.return_code != GRAV_SUCCESS) {
                if (!failed_) {
                    failed_ = true;
                    code_ = e.return_code;
                    msg_ = e.traceback ? e.traceback : "snapshot write failed";
                }
                free_traceback(&e);
            }
            s.busy = false;
            cv_.notify_all();
        }
    }

    ErrorStatus failure() const
    {
        return GS_RAISE(code_, "snapshot writer: %s", msg_.c_str());
    }

    const OutputParam *op_;
    const System *system_;
    Slot slots_[2];
    std::deque<int> queue_;
    std::mutex mu_;
    std::condition_variable cv_;
    bool stop_ = false, failed_ = false;
    int code_ = GRAV_SUCCESS;
    std::string msg_;
    std::thread thread_;
};

OutputContext::OutputContext() = default;
OutputContext::~OutputContext() = default;

ErrorStatus OutputContext::take(int n, const double *d_x, const double *d_v, const int *d_ids,
                                const double *d_m, const int *d_cnt, cudaStream_t s, double t,
                                double dt)
{
    if (!writer) writer.reset(new SnapshotWriter(op, system));
    GS_TRY(writer->take(op->output_count_, n, d_x, d_v, d_ids, d_m, d_cnt, s, t, dt));
    ++op->output_count_;
    next_time = op->output_count_ * op->output_interval;
    return ok();
}

ErrorStatus OutputContext::finish()
{
    if (writer) GS_TRY(writer->finish());
    return ok();
}

}  // namespace gs

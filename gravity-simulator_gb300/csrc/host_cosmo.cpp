// host_cosmo.cpp -- the cosmological entry points of grav_sim's C ABI:
// acceleration_PM (src/acceleration_PM.c:274-391), leapfrog_cosmology
// (src/integrator_cosmology_leapfrog.c:24-255), launch_cosmological_simulation
// (src/grav_sim.c:140-255) and their host helpers (src/cosmology.c,
// src/system.c:121-243, :1337-1375).  The particle-mesh force and the
// integration run on the GPU (k_pm.cu); this file keeps the reference's
// argument checks, in its order and with its messages.
#include "gs_internal.h"

#include <cmath>

extern "C" {

// src/system.c:121-141
CosmologicalSystem get_new_cosmological_system(void)
{
    CosmologicalSystem s;
    s.num_particles = 0;
    s.particle_ids = nullptr;
    s.x = nullptr;
    s.v = nullptr;
    s.m = nullptr;
    s.h = -1.0;
    s.omega_m = -1.0;
    s.omega_lambda = -1.0;
    s.omega_k = 0.0;
    s.box_center[0] = 0.0;
    s.box_center[1] = 0.0;
    s.box_center[2] = 0.0;
    s.box_width = -1.0;
    s.unit_mass = 1.0;
    s.unit_length = 1.0;
    s.unit_time = 1.0;
    return s;
}

// src/system.c:174-242
ErrorStatus finalize_cosmological_system(CosmologicalSystem *system)
{
    if (!system) return GS_RAISE(GRAV_POINTER_ERROR, "System is NULL");
    if (system->num_particles <= 0)
        return GS_RAISE(GRAV_VALUE_ERROR, "Number of particles must be positive. Got: %d",
                        system->num_particles);
    if (!system->particle_ids)
        return GS_RAISE(GRAV_POINTER_ERROR, "System array particle_ids is NULL");
    if (!system->x) return GS_RAISE(GRAV_POINTER_ERROR, "System array x is NULL");
    if (!system->v) return GS_RAISE(GRAV_POINTER_ERROR, "System array v is NULL");
    if (!system->m) return GS_RAISE(GRAV_POINTER_ERROR, "System array m is NULL");
    if (system->h <= 0.0)
        return GS_RAISE(GRAV_VALUE_ERROR, "Hubble parameter system->h must be positive. Got: %g",
                        system->h);
    if (system->omega_m <= 0.0)
        return GS_RAISE(GRAV_VALUE_ERROR, "omega_m must be positive. Got: %g", system->omega_m);
    if (system->omega_lambda <= 0.0)
        return GS_RAISE(GRAV_VALUE_ERROR, "omega_lambda must be positive. Got: %g",
                        system->omega_lambda);
    if (system->box_width <= 0.0)
        return GS_RAISE(GRAV_VALUE_ERROR, "Box width must be positive. Got: %g", system->box_width);
    return gs::ok();
}

// src/cosmology.c:5-11
double compute_omega_k(double omega_m, double omega_lambda)
{
    return 1.0 - omega_m - omega_lambda;
}

// src/cosmology.c:13-26
double compute_da(double a, double H0, double omega_m, double omega_lambda)
{
    const double omega_k = compute_omega_k(omega_m, omega_lambda);
    return H0 * a * std::sqrt(omega_lambda + omega_m / (a * a * a) + omega_k / (a * a));
}

// src/system.c:1337-1375 on host arrays.
void set_periodic_boundary_conditions(CosmologicalSystem *system)
{
    const int n = system->num_particles;
    double *x = system->x;
    const double *c = system->box_center;
    const double bw = system->box_width;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < 3; ++j) {
            const double p = x[i * 3 + j] - c[j];
            if (p < -bw) {
                x[i * 3 + j] = ((int)(p / bw) % 2 != 0) ? std::fmod(p, bw) + bw : std::fmod(p, bw);
                x[i * 3 + j] += c[j];
            } else if (p > bw) {
                x[i * 3 + j] = ((int)(p / bw) % 2 != 0) ? std::fmod(p, bw) - bw : std::fmod(p, bw);
                x[i * 3 + j] += c[j];
            }
        }
}

ErrorStatus acceleration_PM(double *a, int num_particles, const double *x, const double *m,
                            const double *box_center, double box_width, double H0,
                            double omega_m, double mean_bkg_density, int pm_grid_size,
                            double scale_factor)
{
    return gs::pm_acceleration_host(a, num_particles, x, m, box_center, box_width, H0, omega_m,
                                    mean_bkg_density, pm_grid_size, scale_factor);
}

ErrorStatus leapfrog_cosmology(CosmologicalSystem *system, OutputParam *output_param,
                               SimulationStatus *simulation_status, Settings *settings, double dt,
                               double a_begin, double a_final, int pm_grid_size)
{
    if (!system || !output_param || !simulation_status || !settings)
        return GS_RAISE(GRAV_POINTER_ERROR, "NULL argument");
    // Cosmological snapshots are HDF5 only (src/output.c:294-337).
    if (output_param->method == OUTPUT_METHOD_CSV)
        return GS_RAISE(GRAV_VALUE_ERROR,
                        "CSV output method is not supported for cosmological simulation.");
    return gs::pm_leapfrog_cosmology(system, simulation_status, output_param,
                                     settings->is_exit_ptr, dt, a_begin, a_final, pm_grid_size);
}

// src/grav_sim.c:140-255
ErrorStatus launch_cosmological_simulation(CosmologicalSystem *system, OutputParam *output_param,
                                           SimulationStatus *simulation_status,
                                           Settings *settings, double dt, double a_begin,
                                           double a_final, int pm_grid_size)
{
    GS_TRY(finalize_cosmological_system(system));
    if (!output_param) return GS_RAISE(GRAV_POINTER_ERROR, "output_param is NULL");
    if (output_param->method == OUTPUT_METHOD_CSV)
        return GS_RAISE(GRAV_VALUE_ERROR, "CSV output is not supported for cosmological "
                                          "simulations. Please use HDF5 output format.");
    if (!settings) return GS_RAISE(GRAV_POINTER_ERROR, "settings is NULL");
    GS_TRY(gs::output_prepare(output_param, settings));
    if (dt < 0.0) return GS_RAISE(GRAV_VALUE_ERROR, "dt must be non=negative. Got: %g", dt);
    if (a_begin <= 0.0) return GS_RAISE(GRAV_VALUE_ERROR, "a_begin must be positive. Got: %g", a_begin);
    if (a_final <= 0.0) return GS_RAISE(GRAV_VALUE_ERROR, "a_final must be positive. Got: %g", a_final);
    if (a_final < a_begin)
        return GS_RAISE(GRAV_VALUE_ERROR, "a_final must be greater or equal to a_begin. Got: %g, %g",
                        a_begin, a_final);
    if (pm_grid_size <= 0)
        return GS_RAISE(GRAV_VALUE_ERROR, "pm_grid_size must be positive. Got: %d", pm_grid_size);
    if (!simulation_status) return GS_RAISE(GRAV_POINTER_ERROR, "simulation_status is NULL");
    GS_TRY(leapfrog_cosmology(system, output_param, simulation_status, settings, dt, a_begin,
                              a_final, pm_grid_size));
    return gs::ok();
}

// Device time (CUDA events on the run's stream) of the step loop of the
// calling thread's last leapfrog_cosmology / launch_cosmological_simulation,
// and its step count.  Kernels of this library per step: two kicks, the
// drift with the periodic wrap, and five particle-mesh kernels.
int gsgpu_cosmology_last_timing(double *loop_ms, int64_t *steps, int *kernels_per_step)
{
    ErrorStatus st = gs::pm_last_timing(loop_ms, steps);
    if (st.return_code != GRAV_SUCCESS) {
        print_and_free_traceback(&st);
        return st.return_code;
    }
    if (kernels_per_step) *kernels_per_step = 8;
    return 0;
}

}  // extern "C"

// engines_pending.cpp -- factories and entry points of engines not built yet.
#include "gs_internal.h"

#include <cstring>

namespace gs {
std::unique_ptr<Engine> make_massless_engine() { return nullptr; }
std::unique_ptr<Engine> make_barnes_hut_engine(bool) { return nullptr; }
std::unique_ptr<Engine> make_learned_engine() { return nullptr; }
}  // namespace gs

extern "C" {

ErrorStatus acceleration_barnes_hut(double *a, const System *system,
                                    const AccelerationParam *acceleration_param)
{
    (void)a; (void)system; (void)acceleration_param;
    return GS_RAISE(GRAV_NOT_IMPLEMENTED_ERROR, "Barnes-Hut is not built yet");
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
    (void)octree; (void)system; (void)acceleration_param; (void)box_center; (void)box_width;
    return GS_RAISE(GRAV_NOT_IMPLEMENTED_ERROR, "octree is not built yet");
}

void free_linear_octree(LinearOctree *octree) { (void)octree; }

}  // extern "C"

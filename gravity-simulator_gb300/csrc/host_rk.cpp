// host_rk.cpp -- Butcher tableaus of the embedded Runge-Kutta integrators
// (integrator codes 5-8: Fehlberg 4(5), Dormand-Prince 5(4), Verner 6(5)
// "DVERK", Fehlberg 7(8)), the methods src/integrator_rk_embedded.c:79-325
// uses, with its (power, power_test) pairs.
//
// The coefficients are the published rationals, converted to double by one
// IEEE division each: for every entry that rounding equals the rounding of
// the quotient formed in long double and then narrowed, so the doubles are
// those the reference computes on x86-64 and on aarch64.
#include "gs_internal.h"

namespace gs {
namespace {

struct Q {
    int p, q;
};

// Lower triangle of the stage matrix, row s = 1..S-1 holding a[s][0..s-1].
const Q kF45A[] = {{1, 4},
                   {3, 32}, {9, 32},
                   {1932, 2197}, {-7200, 2197}, {7296, 2197},
                   {439, 216}, {-8, 1}, {3680, 513}, {-845, 4104},
                   {-8, 27}, {2, 1}, {-3544, 2565}, {1859, 4104}, {-11, 40}};
const Q kF45B[] = {{25, 216}, {0, 1}, {1408, 2565}, {2197, 4104}, {-1, 5}, {0, 1}};
const Q kF45E[] = {{16, 135}, {0, 1}, {6656, 12825}, {28561, 56430}, {-9, 50}, {2, 55}};

const Q kDPA[] = {{1, 5},
                  {3, 40}, {9, 40},
                  {44, 45}, {-56, 15}, {32, 9},
                  {19372, 6561}, {-25360, 2187}, {64448, 6561}, {-212, 729},
                  {9017, 3168}, {-355, 33}, {46732, 5247}, {49, 176}, {-5103, 18656},
                  {35, 384}, {0, 1}, {500, 1113}, {125, 192}, {-2187, 6784}, {11, 84}};
const Q kDPB[] = {{35, 384}, {0, 1}, {500, 1113}, {125, 192}, {-2187, 6784}, {11, 84}, {0, 1}};
const Q kDPE[] = {{5179, 57600}, {0, 1},        {7571, 16695}, {393, 640},
                  {-92097, 339200}, {187, 2100}, {1, 40}};

const Q kV65A[] = {{1, 6},
                   {4, 75}, {16, 75},
                   {5, 6}, {-8, 3}, {5, 2},
                   {-165, 64}, {55, 6}, {-425, 64}, {85, 96},
                   {12, 5}, {-8, 1}, {4015, 612}, {-11, 36}, {88, 255},
                   {-8263, 15000}, {124, 75}, {-643, 680}, {-81, 250}, {2484, 10625}, {0, 1},
                   {3501, 1720}, {-300, 43}, {297275, 52632}, {-319, 2322}, {24068, 84065},
                   {0, 1}, {3850, 26703}};
const Q kV65B[] = {{3, 40}, {0, 1}, {875, 2244}, {23, 72}, {264, 1955}, {0, 1}, {125, 11592},
                   {43, 616}};
const Q kV65E[] = {{13, 160}, {0, 1}, {2375, 5984}, {5, 16}, {12, 85}, {3, 44}, {0, 1}, {0, 1}};

const Q kF78A[] = {
    {2, 27},
    {1, 36}, {1, 12},
    {1, 24}, {0, 1}, {1, 8},
    {5, 12}, {0, 1}, {-25, 16}, {25, 16},
    {1, 20}, {0, 1}, {0, 1}, {1, 4}, {1, 5},
    {-25, 108}, {0, 1}, {0, 1}, {125, 108}, {-65, 27}, {125, 54},
    {31, 300}, {0, 1}, {0, 1}, {0, 1}, {61, 225}, {-2, 9}, {13, 900},
    {2, 1}, {0, 1}, {0, 1}, {-53, 6}, {704, 45}, {-107, 9}, {67, 90}, {3, 1},
    {-91, 108}, {0, 1}, {0, 1}, {23, 108}, {-976, 135}, {311, 54}, {-19, 60}, {17, 6}, {-1, 12},
    {2383, 4100}, {0, 1}, {0, 1}, {-341, 164}, {4496, 1025}, {-301, 82}, {2133, 4100}, {45, 82},
    {45, 164}, {18, 41},
    {3, 205}, {0, 1}, {0, 1}, {0, 1}, {0, 1}, {-6, 41}, {-3, 205}, {-3, 41}, {3, 41}, {6, 41},
    {0, 1},
    {-1777, 4100}, {0, 1}, {0, 1}, {-341, 164}, {4496, 1025}, {-289, 82}, {2193, 4100}, {51, 82},
    {33, 164}, {19, 41}, {0, 1}, {1, 1}};
const Q kF78B[] = {{41, 840}, {0, 1}, {0, 1}, {0, 1},   {0, 1},    {34, 105}, {9, 35},
                   {9, 35},   {9, 280}, {9, 280}, {41, 840}, {0, 1}, {0, 1}};
const Q kF78E[] = {{0, 1},  {0, 1},   {0, 1},   {0, 1}, {0, 1},    {34, 105}, {9, 35},
                   {9, 35}, {9, 280}, {9, 280}, {0, 1}, {41, 840}, {41, 840}};

RkTableau build(int stages, int power, int power_test, const Q *a, const Q *b, const Q *e)
{
    RkTableau t{};
    t.stages = stages;
    t.power = power;
    t.power_test = power_test;
    int k = 0;
    for (int s = 1; s < stages; ++s)
        for (int i = 0; i < s; ++i, ++k) t.a[s][i] = (double)a[k].p / (double)a[k].q;
    for (int s = 0; s < stages; ++s) {
        t.b[s] = (double)b[s].p / (double)b[s].q;
        t.b_hat[s] = (double)e[s].p / (double)e[s].q;
    }
    return t;
}

}  // namespace

const RkTableau *rk_tableau(int integrator)
{
    static const RkTableau t[4] = {build(6, 4, 5, kF45A, kF45B, kF45E),
                                   build(7, 5, 4, kDPA, kDPB, kDPE),
                                   build(8, 6, 7, kV65A, kV65B, kV65E),
                                   build(13, 7, 8, kF78A, kF78B, kF78E)};
    return (integrator >= INTEGRATOR_RKF45 && integrator <= INTEGRATOR_RKF78)
               ? &t[integrator - INTEGRATOR_RKF45]
               : nullptr;
}

}  // namespace gs

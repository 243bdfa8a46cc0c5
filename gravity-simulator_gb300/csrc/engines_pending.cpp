// engines_pending.cpp -- factories of engines not built yet.
#include "gs_internal.h"

namespace gs {
std::unique_ptr<Engine> make_massless_engine() { return nullptr; }
std::unique_ptr<Engine> make_learned_engine() { return nullptr; }
}  // namespace gs

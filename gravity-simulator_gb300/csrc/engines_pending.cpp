// engines_pending.cpp -- factories of engines not built yet.
#include "gs_internal.h"

namespace gs {
std::unique_ptr<Engine> make_learned_engine() { return nullptr; }
}  // namespace gs

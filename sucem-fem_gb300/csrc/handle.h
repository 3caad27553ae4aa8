// Definition of the opaque C-ABI handle.
#pragma once
#include "space.h"

struct sucem_space {
  sucem::Space s;
};

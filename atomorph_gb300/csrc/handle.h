// The opaque handle behind am_morph* (include/atomorph_gb300.h).
#pragma once

#include "engine.h"

struct am_morph {
    amg::Engine e;
};

// Device state of the fluid solver (k_fluid.cu) shared with the morph's
// fluid path (k_fluid_morph.cu).
#pragma once

#include "common.cuh"

namespace amg {

// Particle fields, FP32 structure of arrays [kFlFields][n]: position,
// velocity, gravity (attractor) point, freedom-radius multiplier, strength,
// ideal colour R G B A and current colour r g b a.
enum { PX, PY, PU, PV, PGX, PGY, PFR, PSTR, PR_, PG_, PB_, PA_, Pr, Pg, Pb, Pa, kFlFields };
// Node fields [kFlNode][gsx * gsy].
enum { NM, ND, NGX, NGY, NAX, NAY, NU, NV, NW, NR, NG, NB, NA, kFlNode };

struct FluidDev {
    uint32_t gsx = 0, gsy = 0, n = 0;
    float *P = nullptr;      // [kFlFields][n] in the caller's order
    uint8_t *flags = nullptr;// [n] bit0 active, bit1 mature
    float *G = nullptr;      // [kFlNode][gsx*gsy]
    uint64_t step = 0;
    // solver order (particles sorted by 8x8 cell block) for fluid_run
    float *S = nullptr;      // [kFlFields][n] gathered copy
    uint8_t *sflags = nullptr;
    uint32_t *keys = nullptr, *ids = nullptr, *tkeys = nullptr, *tids = nullptr, *hist = nullptr;
};


}  // namespace amg

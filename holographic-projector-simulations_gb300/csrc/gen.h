// gen.h -- the CLI's generated-data mode on the device (gen.cu).
#pragma once
#include <stddef.h>

#include "io.h"

namespace holo_gen {

// object shapes of the reference (cuda/main.h:9)
constexpr int kShapeLine = 0, kShapeLogLine = 1, kShapeCircle = 2, kShapeDottedCircle = 3;

// init::plane (cuda/init.h:89-158): n points on a lattice of cell centres into
// v_host (3 n doubles); with p.randomize, cuRAND XORWOW jitter from `seed`.
// Returns 0, or -1 on a CUDA / cuRAND failure.
int lattice(double *v_host, size_t n, const holo_io::Plane &p, unsigned int seed);

// init::sparse_plane (cuda/init.h:160-234): the object's n points (u_host, 3 n doubles,
// updated in place: line shapes set x only, the dotted circle keeps point 0).
int object_points(double *u_host, size_t n, int shape, double width, const double *offset,
                  double modulate);

}  // namespace holo_gen

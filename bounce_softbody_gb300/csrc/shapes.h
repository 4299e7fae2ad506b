// Host setup of static world shapes (shapes.cpp).
#pragma once

#include "internal.h"

#include <vector>

namespace b3g {

// Validates the desc's world spheres and shapes and builds their device records (spheres first)
// and the float data meshes and SDFs refer to; `data` members hold offsets into `data` until
// bind_shape_data. Returns nonzero with a message on invalid input.
int build_shapes(const b3g_body_desc* d, std::vector<DevShape>& shapes, std::vector<float>& data, char* msg,
                 size_t cap);
// Turns the data offsets into pointers into the device copy of `data`.
void bind_shape_data(std::vector<DevShape>& shapes, const float* device_data);

} // namespace b3g

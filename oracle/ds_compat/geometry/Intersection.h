// TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT (ds_compat; see core/Globals.h).
//
// cg::Intersection as the reference's patch intersectors use it: `distance`
// is the current best ray distance (in/out), `p` the hit's (u, v)
// (src/Spline_BezierClipping.cu:105-108, src/rt/Primitive.cu:226-239).
#pragma once

#include <limits>
#include "../math/Vector.h"

namespace cg
{

struct Intersection
{
    float distance = std::numeric_limits<float>::infinity();
    Vector<float,2> p {};
    int triangleIndex = 0;
    const void* object = nullptr;
};

} // namespace cg

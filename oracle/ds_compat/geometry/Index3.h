// TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT (ds_compat; see core/Globals.h).
#pragma once
#include "../core/Globals.h"

namespace cg
{

template<typename T> struct Index2 { T x, y; };
template<typename T> struct Index3 { T x, y, z; };

} // namespace cg

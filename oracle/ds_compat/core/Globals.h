// TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// ds_compat: a minimal, from-scratch stand-in for the parts of the un-vendored
// "Ds" library (MachSilva/Ds, .gitmodules:1-3 of the reference) that the
// reference's ray--patch hot path includes.  It lets oracle/build_ref.py
// compile the reference's own sources, unchanged, as host C++ with g++, so
// that the oracle's restatement can be checked against the reference itself.
// The semantics chosen for the Ds types are the ones the oracle states in its
// header: component-wise vector arithmetic, dot products summed left to right,
// length = sqrt(dot), versor/normalize multiply by 1/length, an empty box is
// (+inf, -inf), column-major matrices.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <cmath>

#ifndef HOST
#define HOST __host__
#endif
#ifndef DEVICE
#define DEVICE __device__
#endif

namespace cg
{
} // namespace cg

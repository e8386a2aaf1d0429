// TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// Force-included (g++ -include) before every reference source compiled by
// oracle/build_ref.py.  The reference's .cu files also hold device-only
// functions (the GPU clip and subdivision loops); g++ compiles their bodies as
// host code although nothing on the host calls them.  These host stand-ins
// for the few device intrinsics in those bodies exist only so that they
// compile: __trap aborts, __builtin_assume (a hint) is dropped, and the bit operations are the plain definitions
// (count leading zeros, bit reversal).
#pragma once

#include <cstdint>
#include <cstdlib>
#include <cuda_runtime.h>
#include <cuda_fp16.h>

inline void __trap() { std::abort(); }
// An optimisation hint of nvcc and clang; g++ has no such builtin.
#if !defined(__clang__)
#define __builtin_assume(x) static_cast<void>(0)
#endif
inline int __clz(unsigned x) { return x ? __builtin_clz(x) : 32; }
inline int __clz(int x) { return __clz(unsigned(x)); }
inline unsigned __brev(unsigned x)
{
    unsigned r = 0;
    for (int i = 0; i < 32; i++) { r = (r << 1) | (x & 1u); x >>= 1; }
    return r;
}
inline int __clzll(long long x) { return x ? __builtin_clzll((unsigned long long)x) : 64; }
inline unsigned long long __brevll(unsigned long long x)
{
    unsigned long long r = 0;
    for (int i = 0; i < 64; i++) { r = (r << 1) | (x & 1ull); x >>= 1; }
    return r;
}

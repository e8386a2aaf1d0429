// TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT (ds_compat; see core/Globals.h).
#pragma once

#include <chrono>

namespace cg
{

// Elapsed wall-clock time since start(), in milliseconds.
class Stopwatch
{
public:
    void start() { _t0 = std::chrono::steady_clock::now(); }
    double time() const
    {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - _t0).count();
    }

private:
    std::chrono::steady_clock::time_point _t0 = std::chrono::steady_clock::now();
};

} // namespace cg

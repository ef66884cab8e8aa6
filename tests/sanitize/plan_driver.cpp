// Host-code driver run under AddressSanitizer and UndefinedBehaviorSanitizer
// (tests/test_host_sanitizers.py): builds the ADI line plan (the FP64 host
// precomputation of the partitioned Thomas solve, hal-cpp_gb300/csrc/
// adi_plan.cpp) for every line-length class, rate range and end condition,
// and checks each plan's self-check and array sizes.  Any out-of-bounds
// access, overflow or invalid shift aborts the run.
#include "adi_plan.h"

#include <cmath>
#include <cstdio>

int main()
{
    using namespace halcuda;
    const int32_t lengths[] = {1, 2, 3, 4, 31, 32, 33, 63, 64, 65, 100, 255, 256, 257, 1000, 1024, 2048, 4095, 4096};
    const double rates[] = {1e-3, 0.3, 1.0, 5.0, 100.0};
    const int ends[] = {kEndsZeroFlux, kEndsDirichlet, kEndsPeriodic};
    int plans = 0;
    for (int32_t L : lengths)
    {
        for (double r : rates)
        {
            for (int e : ends)
            {
                AdiLinePlanHost h;
                if (!BuildAdiLinePlan(L, r, e, h))
                {
                    std::printf("plan L=%d r=%g ends=%d: not built\n", L, r, e);
                    return 1;
                }
                const size_t P = static_cast<size_t>((L + kAdiM - 1) / kAdiM);
                const bool sizes = h.L == L && static_cast<size_t>(h.P) == P &&
                                   h.coef.size() == static_cast<size_t>(3 * kCoefCount * kAdiM) &&
                                   h.gband.size() == (P > 1 ? (P - 1) * static_cast<size_t>(2 * h.B + 1) : 0) &&
                                   (e != kEndsPeriodic || h.zsm.size() == static_cast<size_t>(L));
                if (!sizes || !(h.selfCheck < 1e-5) || !std::isfinite(h.selfCheck))
                {
                    std::printf("plan L=%d r=%g ends=%d: sizes %d, self-check %g\n", L, r, e, sizes ? 1 : 0,
                                h.selfCheck);
                    return 1;
                }
                plans++;
            }
        }
    }
    // lengths outside [1, 4096] are refused
    AdiLinePlanHost h;
    if (BuildAdiLinePlan(0, 1.0, kEndsZeroFlux, h) || BuildAdiLinePlan(4097, 1.0, kEndsZeroFlux, h))
    {
        std::printf("out-of-range length accepted\n");
        return 1;
    }
    std::printf("ok %d plans\n", plans);
    return 0;
}

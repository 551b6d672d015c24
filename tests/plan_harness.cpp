// Host build of the step kernel's work-list planner (poe2d_plan.h) for
// tests/test_plan.py: the same header the library compiles.
#include <stdint.h>

#include <vector>

#include "poe2d_plan.h"

extern "C" int balanced_order_c(const uint8_t *edge, int n, int slots, int *out)
{
    const std::vector<uint8_t> e(edge, edge + n);
    const std::vector<int> o = poe::balanced_order(e, slots);
    for (int i = 0; i < (int)o.size(); ++i) out[i] = o[(size_t)i];
    return (int)o.size();
}

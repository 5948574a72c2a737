// Single-node stand-in for get_mempolicy (include/numa_helper.hpp:262-267).
// Test infrastructure for building the reference baseline.
#pragma once
#define MPOL_F_NODE (1 << 0)
#define MPOL_F_ADDR (1 << 1)
static inline long get_mempolicy(int *mode, unsigned long *, unsigned long, void *, unsigned long)
{
    if (mode) *mode = 0;
    return 0;
}

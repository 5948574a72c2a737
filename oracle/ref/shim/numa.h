// Minimal single-node stand-in for the libnuma calls the reference makes
// (include/numa_helper.hpp, include/memory.hpp, include/sysinfo.hpp).  Node
// allocations map anonymous, zero-filled pages like numa_alloc_onnode does.
// Test infrastructure for building the reference baseline; not part of the
// engine.
#pragma once
#include <stddef.h>
#include <sys/mman.h>

struct bitmask {
    unsigned long size;
    unsigned long *maskp;
};

static inline int numa_available(void) { return 0; }
static inline int numa_num_configured_nodes(void) { return 1; }
static inline struct bitmask *numa_parse_nodestring(const char *)
{
    static struct bitmask b = {0, 0};
    return &b;
}
static inline void numa_set_interleave_mask(struct bitmask *) {}
static inline int numa_run_on_node(int) { return 0; }
static inline void *ptw_numa_map(size_t size)
{
    void *p = mmap(NULL, size ? size : 1, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    return p == MAP_FAILED ? NULL : p;
}
static inline void *numa_alloc_onnode(size_t size, int) { return ptw_numa_map(size); }
static inline void *numa_alloc_interleaved(size_t size) { return ptw_numa_map(size); }
static inline void numa_free(void *p, size_t size) { munmap(p, size ? size : 1); }
static inline void numa_tonode_memory(void *, size_t, int) {}

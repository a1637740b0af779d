/* scatter_oracle.h — CPU restatement of mallocMC's Scatter creation policy.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle). It is the checker for the CUDA heap in
 * mallocmc_gb300/: tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it; the product path never does.
 *
 * It restates, in plain C, the algorithm of the reference's
 *   src/include/mallocMC/creationPolicies/Scatter.hpp      (heap, malloc, free, slots)
 *   src/include/mallocMC/device_allocator.hpp:72-106       (malloc/free/getAvailableSlots glue)
 *   src/include/mallocMC/alignmentPolicies/Shrink.hpp:132-137 (padding)
 *   src/include/mallocMC/distributionPolicies/XMallocSIMD.hpp:118-176 (one-lane case)
 * with the reference's CPU-backend semantics (mallocMC_utils.hpp:72-136):
 * warpSize = 1, laneid = warpid = smid = 0, ballot/activemask = 1. Under these
 * semantics XMallocSIMD never coalesces (XMallocSIMD.hpp:134-138), so the
 * distribution policy is the identity here.
 *
 * Pinning: every function is checked against tests/golden fixtures produced
 * by the reference itself (oracle/ref_harness.cpp on alpaka CPU-serial).
 *
 * The heap lives in a host buffer with the reference's byte layout
 * (Scatter.hpp:999-1019): [Page x numpages][PTE{chunksize,count,bitmask} x
 * numpages][u32 region x numregions]. All atomics are GCC __atomic builtins so
 * the same code also runs concurrently (the multi-threaded CPU baseline).
 */
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oc_config
{
    uint32_t pagesize;        /* Scatter.hpp:60 */
    uint32_t regionsize;      /* Scatter.hpp:67 */
    uint32_t wastefactor;     /* Scatter.hpp:69 */
    uint32_t resetfreedpages; /* Scatter.hpp:77 */
    uint64_t accessblocksize; /* Scatter.hpp:65 */
    uint32_t hashingK;        /* Scatter.hpp:82-85 */
    uint32_t hashingDistMP;
    uint32_t hashingDistWP;
    uint32_t hashingDistWPRel;
    uint32_t dataAlignment;   /* Shrink<dataAlignment>; 0 selects AlignmentPolicies::Noop */
    uint32_t reference_quirks; /* 1: keep the reference's exact-pagesize and page-based underflow quirks */
} oc_config;

typedef struct oc_heap oc_heap;

/* error codes */
#define OC_OK 0
#define OC_ERR_CONFIG 1
#define OC_ERR_NOMEM 2

/* Create a heap over a host buffer of memsize bytes (the oracle allocates it).
 * Mirrors Allocator::alloc (allocator.hpp:136-159) + Scatter::initHeap/initDeviceFunction
 * (Scatter.hpp:956-1096). Returns OC_ERR_CONFIG where the reference would divide
 * by zero (heap smaller than one access block, Scatter.hpp:991-993). */
int oc_heap_create(const oc_config* cfg, uint64_t memsize, oc_heap** out);
void oc_heap_destroy(oc_heap* h);

/* DeviceAllocator::malloc / free (device_allocator.hpp:72-88) with CPU ids. */
void* oc_malloc(oc_heap* h, uint64_t bytes);
void oc_free(oc_heap* h, void* p);
/* Allocator::getAvailableSlots (allocator.hpp:227-233 -> Scatter.hpp:1235-1295). */
uint32_t oc_available_slots(oc_heap* h, uint64_t slotSize);
/* handle.getAvailableSlots (device_allocator.hpp:98-106 -> Scatter.hpp:1311-1352), one thread. */
uint32_t oc_available_slots_accelerator(oc_heap* h, uint64_t slotSize);

/* Layout/introspection */
uint8_t* oc_pool(oc_heap* h);
uint32_t oc_numpages(oc_heap* h);
uint32_t oc_accessblocks(oc_heap* h);
uint32_t oc_numregions(oc_heap* h);
uint32_t oc_max_on_page_masks(oc_heap* h);
uint32_t oc_hierarchy_threshold(oc_heap* h);
/* header words: [0]=firstFreePageBased [1]=firstfreeblock [2]=pagebasedMutex */
void oc_header(oc_heap* h, uint32_t out[3]);
/* copy the PTE array as numpages x {chunksize,count,bitmask} */
void oc_snapshot_ptes(oc_heap* h, uint32_t* out3);
void oc_snapshot_regions(oc_heap* h, uint32_t* out);
/* copy the last maxOnPageMasks words of every page (numpages x maxOnPageMasks) */
void oc_snapshot_masks(oc_heap* h, uint32_t* out);
/* load PTE + region + mask state (same formats) into the heap, e.g. a GPU snapshot */
void oc_load_state(oc_heap* h, const uint32_t* ptes3, const uint32_t* regions, const uint32_t* masks);

/* Run an op program in one thread: ops[i] = {kind, arg}; kind 'm' malloc(arg),
 * 'f' free the block returned by op number arg, 's' host slots(arg), 'd'
 * accelerator slots(arg). out[i] = pool offset (malloc; -1 for null), slot
 * count, or 0 (the same program format as the C ABI's mmc_run_program). */
void oc_run_program(oc_heap* h, const uint8_t* kinds, const uint64_t* args, int64_t n, int64_t* out);

/* Seeded request sizes shared with the CUDA workloads (SplitMix64 finaliser of
 * a counter; identical in C, CUDA and numpy). */
uint64_t oc_mix64(uint64_t seed, uint64_t a, uint64_t b);

/* Multi-threaded stress run with the reference CPU-backend semantics: `workers`
 * host threads pull virtual GPU threads (alpaka CPU blocks of one thread) from
 * a shared counter; each virtual thread does `rounds` x {malloc(size drawn in
 * [lo, hi] step `step`), write a u64 pattern, verify it, free}. Returns the
 * malloc+free pairs completed; *nulls and *bad count null returns and pattern
 * mismatches; *seconds is the wall time. */
uint64_t oc_run_stress(oc_heap* h, uint64_t vthreads, uint32_t rounds, uint64_t seed, uint32_t lo, uint32_t hi,
                       uint32_t step, int workers, uint64_t* nulls, uint64_t* bad, double* seconds);

/* Size of request i of the fragmentation workload: with probability
 * large_permille / 1000 log-uniform in [large_lo, large_hi], else uniform in
 * [small_lo, small_hi] (identical draw in C, CUDA and numpy). */
uint32_t oc_frag_size(uint64_t seed, uint64_t i, uint32_t small_lo, uint32_t small_hi, uint32_t large_lo,
                      uint32_t large_hi, uint32_t large_permille);

/* The fragmentation workload run serially: phase 1 allocates requests 0, 1, ...
 * until the first NULL; then a seeded half of the live blocks (a Fisher-Yates
 * permutation of the live list, first half) is freed; phase 2 allocates
 * requests first_null+1, ... until the next NULL. out[0..5] = {phase-1
 * allocations, phase-1 live bytes, freed blocks, phase-2 allocations, final
 * live bytes, seconds x 1e6}. Live bytes count requested sizes. */
void oc_run_fragmentation(oc_heap* h, uint64_t seed, uint32_t small_lo, uint32_t small_hi, uint32_t large_lo,
                          uint32_t large_hi, uint32_t large_permille, uint64_t* out);

#ifdef __cplusplus
}
#endif

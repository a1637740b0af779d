/* mallocmc_gb300.h — C ABI of the GB300 (sm_103a) ScatterAlloc heap.
 *
 * A heap is a device-resident ScatterAlloc pool (pages, page-table entries,
 * region fill counters) plus a small device header. Host code creates and
 * queries it through these functions; kernels allocate from it through the
 * device functions in <mallocMC/scatter_device.cuh> using the POD
 * mmc_device_handle, passed to kernels by value.
 *
 * Each entry point names the reference interface it replaces (paths relative
 * to the mallocMC project root). Conventions: every function returns an
 * mmc_status (0 = success); mmc_last_error() gives a message for the calling
 * thread's last failure. Host calls on one heap are stream-ordered and not
 * thread-safe (the reference's queue semantics); device calls are fully
 * concurrent. No exception crosses this boundary.
 */
#ifndef MALLOCMC_GB300_H
#define MALLOCMC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MMC_VERSION_MAJOR 2
#define MMC_VERSION_MINOR 6
#define MMC_VERSION_PATCH 0

typedef enum mmc_status
{
    MMC_OK = 0,
    MMC_ERR_CONFIG = 1,  /* invalid configuration (e.g. heap smaller than one access block) */
    MMC_ERR_CUDA = 2,    /* a CUDA runtime call failed */
    MMC_ERR_TIMEOUT = 3, /* a bounded device wait gave up (see mmc_heap_error) */
    MMC_ERR_OOM = 4,     /* the pool could not be allocated */
    MMC_ERR_ARG = 5      /* bad argument (null pointer, size out of range) */
} mmc_status;

/* Distribution policies (src/include/mallocMC/distributionPolicies/). */
#define MMC_DIST_NOOP 0        /* DistributionPolicies::Noop (Noop.hpp:46-72) */
#define MMC_DIST_XMALLOCSIMD 1 /* DistributionPolicies::XMallocSIMD (XMallocSIMD.hpp:76-185) */

/* OOM policies (src/include/mallocMC/oOMPolicies/). */
#define MMC_OOM_RETURNNULL 0 /* OOMPolicies::ReturnNull (ReturnNull.hpp:44-57) */
#define MMC_OOM_FLAG 1       /* BadAllocException's device branch without the trap: sets MMC_DEVERR_OOM, returns NULL */

/* Device error bits reported by mmc_heap_error. */
#define MMC_DEVERR_TIMEOUT 0x1u  /* the page-based mutex wait hit its iteration bound */
#define MMC_DEVERR_BADFREE 0x2u  /* free of a pointer outside the heap or on an unformatted page */
#define MMC_DEVERR_OOM 0x4u      /* an allocation failed under MMC_OOM_FLAG */
#define MMC_DEVERR_BADCMD 0x8u   /* a serving tick skipped a command (slot beyond the table, unknown kind,
                                    an admission longer than a slot's chunks hold)
                                    or cut a queue length beyond the queue's capacity */
#define MMC_DEVERR_PAGEBASED 0x10u /* a request above a page in a kernel built without the multi-page path
                                      (mmc::dev::SmallRequests: a batch whose job sizes fit a page, for one) */

/* Device event counters (mmc_heap_stats); maintained only when the library is
 * built with MMC_DEVICE_STATS, zero otherwise. */
#define MMC_STAT_CHUNKED 0       /* chunked allocations started (allocChunked calls) */
#define MMC_STAT_FIRST_PAGE 1    /* ... served by the walk's first page */
#define MMC_STAT_WALK_PAGES 2    /* further pages tried by the walk */
#define MMC_STAT_REGION_FAIL 3   /* regions walked without success (region counter bumps) */
#define MMC_STAT_REGION_SKIP 4   /* regions skipped as 3/4 full (pass 0) or full */
#define MMC_STAT_SIZE_MISMATCH 5 /* pages tried whose chunk size did not fit the request */
#define MMC_STAT_PAGE_FULL 6     /* pages tried whose chunks were all taken */
#define MMC_STAT_CHUNKED_FAIL 7  /* chunked allocations that returned NULL */
#define MMC_STAT_PAGE_BASED 8    /* multi-page allocations started */
#define MMC_STAT_PAGE_SCAN 9     /* page-table words read by concurrent multi-page searches */
#define MMC_STAT_PAGE_LOST 10    /* runs a concurrent multi-page search lost to another claim */
#define MMC_STAT_PAGE_BASED_FAIL 11 /* concurrent multi-page allocations that returned NULL */
#define MMC_STAT_PAGE_SCAN_USED 12 /* free-page bitmap words those searches read with no free page */
#define MMC_STAT_COUNT 16

/* Heap configuration: the template parameters of Scatter<HeapConfig, HashConfig>
 * (creationPolicies/Scatter.hpp:56-85, 124-207), XMallocSIMD<Config> and
 * Shrink<Config> (alignmentPolicies/Shrink.hpp:62-65) as runtime values. */
typedef struct mmc_config
{
    uint32_t pagesize;         /* bytes per page (>= 1024, multiple of 16) */
    uint32_t regionsize;       /* pages per region */
    uint32_t wastefactor;      /* chunk reuse bound: chunksize <= wastefactor * bytes */
    uint32_t resetfreedpages;  /* 1: a fully freed page forgets its chunk size */
    uint64_t accessblocksize;  /* bytes per access block (heap must hold at least one) */
    uint32_t hashingK;         /* page-hash multiplier of the request size */
    uint32_t hashingDistMP;    /* page-hash multiplier of the SM id */
    uint32_t hashingDistWP;    /* page-hash multiplier of the warp id */
    uint32_t hashingDistWPRel; /* page-hash multiplier of warp id x relative size */
    uint32_t dataAlignment;    /* Shrink alignment (power of two); 0 or 1 = AlignmentPolicies::Noop */
    uint32_t distribution;     /* MMC_DIST_* */
    uint32_t oom_policy;       /* MMC_OOM_* */
    uint32_t reference_quirks; /* 1: keep the reference's exact-pagesize free and page-based
                                  underflow behaviour bit for bit (default); 0: fixed */
} mmc_config;

/* Fill *cfg with the reference defaults: DefaultScatterConfig/DefaultScatterHashingParams
 * (Scatter.hpp:56-85), XMallocSIMD, ReturnNull, Shrink<16>. */
void mmc_config_default(mmc_config* cfg);

/* Device-resident mutable header words (one per heap, 128-byte separated). */
typedef struct mmc_heap_state mmc_heap_state;

/* Everything a kernel needs to allocate, passed by value (kernel parameter
 * space). The reference's AllocatorHandleImpl holds a pointer to the device
 * allocator object (mallocMC_allocator_handle.hpp:35-63); here the immutable
 * fields travel with the handle and only the mutable words live in memory. */
typedef struct mmc_device_handle
{
    mmc_heap_state* state;
    char* pages;         /* page i starts at pages + i * pagesize (= pool start) */
    uint32_t* chunksize; /* per-page chunk size (page-table entry word 0) */
    uint32_t* count;     /* per-page fill count (word 1) */
    uint32_t* bitmask;   /* per-page chunk / segment bitmask (word 2) */
    uint32_t* regions;   /* per-region fill counters */
    uint32_t* freemap;   /* free-page bitmap: bit (i & 31) of word i >> 5 is set while page i
                            has chunk size 0 (heap-owned, outside the pool; read by the
                            concurrent multi-page search) */
    uint32_t numpages;
    uint32_t numregions;
    uint32_t accessblocks;
    uint32_t pagesperblock;
    uint32_t pagesize;
    uint32_t regionsize;
    uint32_t wastefactor;
    uint32_t resetfreedpages;
    uint32_t hashingK;
    uint32_t hashingDistMP;
    uint32_t hashingDistWP;
    uint32_t hashingDistWPRel;
    uint32_t dataAlignment;
    uint32_t distribution;
    uint32_t oom_policy;
    uint32_t reference_quirks;
    uint32_t hierarchyThreshold; /* (pagesize - 8) / 33 */
    uint32_t minChunkSize;       /* (pagesize - 128) / 1024 */
    uint32_t paddedMinChunkSize; /* minChunkSize after alignment padding */
    uint32_t maxOnPageMasks;     /* min(32, ceil(pagesize / (32 * minChunkSize + 4))) */
} mmc_device_handle;

typedef struct mmc_heap mmc_heap;

/* Heap geometry, as initDeviceFunction computes it (Scatter.hpp:956-1049). */
typedef struct mmc_geometry
{
    uint64_t memsize;
    uint32_t numpages;
    uint32_t numregions;
    uint32_t accessblocks;
    uint32_t pagesperblock;
    uint32_t maxOnPageMasks;
    uint32_t hierarchyThreshold;
    uint64_t ptes_offset;    /* byte offset of the page-table arrays from the pool start */
    uint64_t regions_offset; /* byte offset of the region counters from the pool start */
} mmc_geometry;

/* ---------------------------------------------------------------- lifetime */

/* Allocator::Allocator(dev, queue, size) / alloc (allocator.hpp:136-159, 179-183):
 * cudaMalloc a pool of `bytes` on `device` (ReservePoolPolicies::AlpakaBuf,
 * AlpakaBuf.hpp:41-46), align it (Shrink::alignPool, Shrink.hpp:109-130) and
 * initialise the heap on `stream` (Scatter::initHeap, Scatter.hpp:1057-1096).
 * MMC_ERR_CONFIG where the reference would divide by zero (heap smaller than
 * one access block, Scatter.hpp:991-993). */
mmc_status mmc_heap_create(const mmc_config* cfg, size_t bytes, int device, void* stream, mmc_heap** out);

/* Like mmc_heap_create over a caller-owned device pool (not freed by the heap).
 * Scatter::initHeap's nullptr check (Scatter.hpp:1065-1071) is MMC_ERR_ARG. */
mmc_status mmc_heap_create_on_pool(const mmc_config* cfg, void* pool, size_t bytes, int device, void* stream,
                                   mmc_heap** out);

/* ~Allocator / free (allocator.hpp:166-172, 185-189). */
mmc_status mmc_heap_destroy(mmc_heap* heap);

/* Allocator::destructiveResize (allocator.hpp:195-200): drop every allocation,
 * reallocate the pool with `bytes` and initialise it again. */
mmc_status mmc_heap_destructive_resize(mmc_heap* heap, size_t bytes, void* stream);

/* Allocator::getAllocatorHandle / operator AllocatorHandle (allocator.hpp:202-212). */
mmc_status mmc_heap_device_handle(const mmc_heap* heap, mmc_device_handle* out);

/* Allocator::getHeapLocations (allocator.hpp:235-241): the pool start and size. */
mmc_status mmc_heap_locations(const mmc_heap* heap, void** pool, size_t* size);

/* Geometry of the initialised heap (numpages etc., Scatter.hpp:962-1048). */
mmc_status mmc_heap_geometry(const mmc_heap* heap, mmc_geometry* out);

/* Allocator::info (allocator.hpp:214-223) joined with Scatter::classname
 * (Scatter.hpp:1354-1370): writes a NUL-terminated description. */
mmc_status mmc_heap_info(const mmc_heap* heap, char* buf, size_t len);

/* ------------------------------------------------------------- free slots */

/* Allocator::getAvailableSlots (allocator.hpp:227-233 -> Scatter::getAvailableSlotsHost,
 * Scatter.hpp:1235-1295): pads slot_size, counts free slots of that size and
 * waits for the result (*out, an unsigned that wraps like the reference's). */
mmc_status mmc_available_slots(mmc_heap* heap, size_t slot_size, void* stream, unsigned* out);

/* Stream-ordered variant with no host synchronisation: the count is written
 * to *out_dev (device or mapped memory) when the stream reaches it. Safe to
 * capture in a CUDA graph once the heap exists. */
mmc_status mmc_available_slots_async(mmc_heap* heap, size_t slot_size, void* stream, unsigned* out_dev);

/* Free-slot count that allocates nothing, for callers that cannot call
 * cudaMalloc: code inside a framework whose device memory belongs to its own
 * pool allocator, which must not take memory behind the pool's back; a
 * plugin that is handed only a device handle, with no mmc_heap and so no
 * heap-owned scratch; a latency-bound host loop (a serving tick, say) that
 * cannot afford cudaMalloc's implicit device-wide synchronisation. It needs
 * only the handle: the scan's partial sums live in one file-scope __device__
 * array of MMC_NOALLOC_SCAN_BLOCKS_MAX entries (16 bytes each, 32 KiB in all),
 * which every GPU that loads the library holds until the process exits. The
 * count is written to *out_dev (device memory) when `stream` reaches it.
 * scan_blocks = 0 picks 4 x the SM count; more than MMC_NOALLOC_SCAN_BLOCKS_MAX
 * is rejected with MMC_ERR_ARG. The calling thread's current device must be
 * the heap's. The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress), so make that first call before any stream capture;
 * the lookup is repeated on the first call after the device's context changed
 * (after a cudaDeviceReset, say), which should then also come before any
 * capture. Every call shares the array: calls that overlap on the GPU (on two
 * streams, say) race and may return wrong counts. Each call rewrites every
 * entry it reads, so nothing carries over from the last call. This entry
 * point has no counterpart in the reference. */
#define MMC_NOALLOC_SCAN_BLOCKS_MAX 2048
mmc_status mmc_available_slots_noalloc(const mmc_device_handle* handle, size_t slot_size, unsigned scan_blocks,
                                       void* stream, unsigned* out_dev);

/* --------------------------------------------------------- introspection */

/* Device error bits (MMC_DEVERR_*) accumulated since the last clear; waits for
 * `stream`. clear != 0 resets them. */
mmc_status mmc_heap_error(mmc_heap* heap, void* stream, uint32_t* flags, int clear);

/* Device event counters (MMC_STAT_*, MMC_STAT_COUNT values) into out; waits for
 * `stream`; clear != 0 zeroes them. The counters are allocator statistics
 * (pages tried by walks, regions skipped, multi-page words scanned); they have no counterpart
 * in the reference and are maintained only in MMC_DEVICE_STATS builds. */
mmc_status mmc_heap_stats(mmc_heap* heap, void* stream, unsigned long long* out, int clear);

/* Copy the free-page bitmap to a host buffer of (numpages + 31) / 32 words
 * (bit i & 31 of word i >> 5: page i has chunk size 0). Waits for `stream`.
 * No counterpart in the reference (whose multi-page search reads the page
 * table itself). */
mmc_status mmc_snapshot_freemap(mmc_heap* heap, void* stream, uint32_t* words);

/* Copy the metadata to host buffers (each may be NULL): ptes3 = numpages x
 * {chunksize, count, bitmask}; regions = numregions words; masks = numpages x
 * maxOnPageMasks words (the last words of each page); header3 =
 * {firstFreePageBased, firstfreeblock, pagebasedMutex}. Waits for `stream`. */
mmc_status mmc_snapshot_metadata(mmc_heap* heap, void* stream, uint32_t* ptes3, uint32_t* regions, uint32_t* masks,
                                 uint32_t* header3);

/* Message for the calling thread's last failed call ("" if none). */
const char* mmc_last_error(void);

/* ------------------------------------------------------------- workloads
 * Kernels built on the device API (what user kernels do with handle.malloc /
 * handle.free), exported for verification, benchmarking and batching. All
 * pointers are device pointers unless stated; all run on `stream`. */

/* Run an op program in ONE device thread with the reference CPU backend's
 * thread ids (laneid = warpid = smid = 0, warp size 1, mallocMC_utils.hpp:72-136),
 * so pool offsets are bit-identical to the reference's CPU-serial run.
 * kinds[i]: 'm' malloc(args[i]) -> out[i] = pool offset or -1; 'f' free the
 * block returned by op args[i] (an op index); 'd' handle.getAvailableSlots(args[i])
 * -> out[i]; 's' Allocator::getAvailableSlots(args[i]) -> out[i]; other kinds
 * are no-ops. kinds/args/out are device buffers of n entries. */
mmc_status mmc_run_program(mmc_heap* heap, const uint8_t* kinds, const uint64_t* args, int64_t n, int64_t* out,
                           void* stream);

/* Uniform stress (every thread `rounds` x {malloc(size), write a u64 pattern,
 * verify it, free}). Sizes: sizes[r * T + t] (u16, bytes; T = blocks x
 * threads_per_block) if sizes != NULL, else drawn from seed uniformly in
 * {lo, lo+step, ..., hi}. stats (device, 4 x u64, accumulated, caller zeroes):
 * {pairs, nulls, pattern errors, checksum}. At most 2^32 threads and 2^26
 * rounds (MMC_ERR_ARG otherwise). */
typedef struct mmc_stress_params
{
    uint32_t blocks;
    uint32_t threads_per_block;
    uint32_t rounds;
    uint32_t lo, hi, step;
    uint64_t seed;
    uint32_t write_pattern; /* MMC_PATTERN_THREAD or MMC_PATTERN_WARP: how each block is written and verified */
    uint32_t reserved;
} mmc_stress_params;
#define MMC_PATTERN_THREAD 1 /* each thread writes and verifies its own block, 16 bytes per store */
#define MMC_PATTERN_WARP 2   /* the warp writes and verifies its lanes' blocks together, 512 bytes per
                                instruction (threads_per_block must be a multiple of 32) */
mmc_status mmc_run_stress(mmc_heap* heap, const mmc_stress_params* p, const uint16_t* sizes,
                          unsigned long long* stats, void* stream);

/* The plain ScatterAlloc verify workload: every thread mallocs sizes[t] bytes,
 * writes the u32 pattern (t ^ seed), verifies it, frees. offsets[t] receives
 * the pool offset (or -1), errors[0] the count of failed words (both device). */
mmc_status mmc_run_verify(mmc_heap* heap, uint32_t blocks, uint32_t threads_per_block, const uint32_t* sizes,
                          uint32_t seed, int64_t* offsets, unsigned long long* errors, void* stream);

/* Split a verify run into its halves: every thread mallocs sizes[t] and writes
 * its pattern (offsets[t] = pool offset or -1); then the caller inspects the
 * heap; then mmc_run_free_offsets verifies and frees them. */
mmc_status mmc_run_alloc_offsets(mmc_heap* heap, uint32_t blocks, uint32_t threads_per_block, const uint32_t* sizes,
                                 uint32_t seed, int64_t* offsets, void* stream);
mmc_status mmc_run_free_offsets(mmc_heap* heap, uint32_t blocks, uint32_t threads_per_block, const uint32_t* sizes,
                                uint32_t seed, const int64_t* offsets, unsigned long long* errors, void* stream);

/* ReservePoolPolicies::CudaSetLimits::setMemPool (reservePoolPolicies/CudaSetLimits.hpp:59-64):
 * size CUDA's own device heap (cudaLimitMallocHeapSize of the current context)
 * for CreationPolicies::OldMalloc. Must precede the first kernel that calls
 * ::malloc in the process (CUDA refuses later changes). */
mmc_status mmc_oldmalloc_set_heap(size_t bytes, int device);

/* The uniform stress of mmc_run_stress with CreationPolicies::OldMalloc
 * (creationPolicies/OldMalloc.hpp:46-84): ::malloc / ::free on CUDA's device
 * heap, the comparison column for the Scatter heap. Same parameters and stats. */
mmc_status mmc_run_stress_oldmalloc(const mmc_stress_params* p, const uint16_t* sizes, unsigned long long* stats,
                                    void* stream);

/* ------------------------------------------------------- fragmentation
 * Fill until the first NULL, free a chosen half, refill: the heap's fill
 * fraction at out-of-memory under a mix of small and multi-page requests.
 * Request i of a phase has the size oracle/scatter_oracle.h's oc_frag_size
 * describes (with probability large_permille/1000 log-uniform in
 * [large_lo, large_hi], else uniform in [small_lo, small_hi]). Requests are
 * made in waves, one request per thread per wave: in wave w thread t makes
 * request first_request + w*T + t (T threads), so the live mix follows the
 * request order the way a serial run's does, one wave at a time. */
typedef struct mmc_frag_params
{
    uint32_t blocks;
    uint32_t threads_per_block;
    uint64_t seed;
    uint64_t first_request;
    uint32_t small_lo, small_hi;
    uint32_t large_lo, large_hi;
    uint32_t large_permille;
    uint32_t waves; /* waves one mmc_run_fill call launches (one kernel each) */
} mmc_frag_params;

/* Allocate until the first NULL anywhere: a NULL sets a device flag, and the
 * threads of later waves find it set and make no request (the requests of the
 * wave that met the NULL all complete). Each block gets a u64 tag every 4 KiB and at its
 * end, and is appended to the list ptrs/sizes (capacity entries; counters[0]
 * is the list length, counters[1] the live requested bytes, counters[2] the
 * requests made, counters[3] tag errors, counters[4] the stop flag, which the
 * caller zeroes before a phase). */
mmc_status mmc_run_fill(mmc_heap* heap, const mmc_frag_params* p, void** ptrs, uint32_t* sizes, uint64_t capacity,
                        unsigned long long* counters, void* stream);
/* Free the list entries idx[0..n) after checking their tags (counters as above). */
mmc_status mmc_run_free_list(mmc_heap* heap, void** ptrs, uint32_t* sizes, const uint32_t* idx, uint64_t n,
                             unsigned long long* counters, void* stream);
/* Check the tags of every live entry of the list (counters[3] += errors). */
mmc_status mmc_run_verify_list(mmc_heap* heap, void* const* ptrs, const uint32_t* sizes, uint64_t n,
                               unsigned long long* counters, void* stream);

/* ------------------------------------------------------------ batches
 * Many independent allocation jobs of uneven size on one heap. No counterpart
 * in the reference (its callers launch one kernel per job); this is the
 * batched, graph-captured launcher of uneven jobs. */

/* One job: `threads` threads, each running a seeded number of cycles in
 * [min_cycles, max_cycles] of {malloc(size), write a u64 pattern, verify, free};
 * sizes geometric with mean `mean_size` bytes, capped at `max_size`, padded to 16. */
typedef struct mmc_job
{
    uint32_t threads;
    uint32_t item_begin; /* set by mmc_batch_create: first 256-thread work item */
    uint64_t seed;
    uint32_t mean_size;
    uint32_t max_size;
    uint32_t min_cycles;
    uint32_t max_cycles;
} mmc_job;

typedef struct mmc_batch mmc_batch;

/* Upload a job table (host array) for `heap`. persistent_blocks = 0 picks 8 x
 * the SM count. use_graph != 0 captures {counter reset, persistent launch}
 * into a CUDA graph that mmc_batch_run replays. */
mmc_status mmc_batch_create(mmc_heap* heap, const mmc_job* jobs, uint32_t njobs, uint32_t persistent_blocks,
                            int use_graph, void* stream, mmc_batch** out);
/* Run the batch as one persistent launch (the captured graph if any). */
mmc_status mmc_batch_run(mmc_batch* batch, void* stream);
/* Run the same batch as one plain kernel launch per job. */
mmc_status mmc_batch_run_plain(mmc_batch* batch, void* stream);
/* Per-job counters {pairs, nulls, pattern errors, checksum} (njobs x 4) to host. */
mmc_status mmc_batch_stats(mmc_batch* batch, void* stream, unsigned long long* out, int clear);
mmc_status mmc_batch_info(const mmc_batch* batch, uint32_t* total_items, uint32_t* blocks, uint64_t* total_threads);
mmc_status mmc_batch_destroy(mmc_batch* batch);

/* ------------------------------------------------------------ serving
 * A continuous-batching request server on the device-resident heap. No
 * counterpart in the reference. A request grows to final_len 2-byte elements,
 * holding one 16 KiB chunk per 256 elements, and completes by checksumming its
 * elements (sum of value x (index + 1), values a seeded function of seed and
 * index) and freeing its chunks. */
#define MMC_SERVE_FREE 0u
#define MMC_SERVE_LIVE 1u
#define MMC_SERVE_DONE 2u

typedef struct mmc_serve_slot
{
    uint32_t id;
    uint32_t final_len;
    uint32_t len;     /* elements written so far */
    uint32_t nchunks; /* chunks held */
    uint64_t seed;
    uint32_t state;   /* MMC_SERVE_* */
    uint32_t failed;  /* ticks whose chunk allocation failed (retried) */
    uint64_t checksum;
} mmc_serve_slot;

/* One command for the next tick: kind 1 admits request `id` into `slot`;
 * kind 2 releases a completed slot. */
typedef struct mmc_serve_cmd
{
    uint32_t kind;
    uint32_t slot;
    uint32_t id;
    uint32_t final_len;
    uint64_t seed;
} mmc_serve_cmd;

typedef struct mmc_server mmc_server;

/* A server for `slots` concurrent requests of at most max_chunks chunks that
 * grow `step` elements per tick; at most queue_cap commands per tick. The
 * batched tick is captured into a CUDA graph here. */
mmc_status mmc_serve_create(mmc_heap* heap, uint32_t slots, uint32_t max_chunks, uint32_t step, uint32_t queue_cap,
                            mmc_server** out);
/* Mapped pinned host views, which the tick's kernels read and write in place:
 * the command queue and its length (written by the host before a tick), the
 * slot table and the free 16 KiB chunk count (as of the end of the last tick). */
mmc_status mmc_serve_queue(mmc_server* server, mmc_serve_cmd** queue, uint32_t** queue_len, mmc_serve_slot** slots,
                           unsigned** free_chunks);
/* Run one tick and wait for it: batched != 0 replays the captured graph (all
 * live requests in one launch); 0 launches one kernel per live request. The
 * queue is checked first (mmc_serve_check_queue, and every admission's
 * final_len against the max_chunks x 256 elements a slot holds): on
 * MMC_ERR_ARG nothing is launched. The tick's kernels check it again, since
 * the queue is host memory the caller may change at any time: they cut a
 * length beyond the capacity and skip a bad command, and set
 * MMC_DEVERR_BADCMD (mmc_heap_error). */
mmc_status mmc_serve_tick(mmc_server* server, int batched);

/* Host-side check of a command queue before a tick: MMC_ERR_ARG when
 * queue_len exceeds queue_cap, or a command has a kind other than 1 or 2 or a
 * slot >= slots. Needs no GPU. */
mmc_status mmc_serve_check_queue(const mmc_serve_cmd* queue, uint32_t queue_len, uint32_t queue_cap, uint32_t slots);

/* Pipelined ticks: two buffers (b = 0, 1), each with its own command queue and
 * its own results, so the host reads one tick's results and writes the next
 * tick's commands while a tick runs. A tick launched on buffer b applies queue
 * b, grows every live request, and publishes into buffer b: the requests that
 * completed in it (slot and checksum), the chunks the still-live requests will
 * yet take (sum of ceil(final_len / 256) - nchunks) and the free 16 KiB chunk
 * count at its end. */
typedef struct mmc_serve_done
{
    uint32_t slot;
    uint32_t reserved;
    uint64_t checksum;
} mmc_serve_done;

mmc_status mmc_serve_pipeline(mmc_server* server, int buffer, mmc_serve_cmd** queue, uint32_t** queue_len,
                              mmc_serve_done** done, uint32_t** done_len, unsigned long long** remaining,
                              unsigned** free_chunks);
/* Launch the batched tick on `buffer` without waiting for it. Like
 * mmc_serve_tick, it first checks the buffer's queue (mmc_serve_check_queue)
 * and launches nothing on MMC_ERR_ARG. */
mmc_status mmc_serve_launch(mmc_server* server, int buffer);
/* Wait for every tick launched so far. */
mmc_status mmc_serve_wait(mmc_server* server);
/* Wait for the last tick launched on `buffer` (ticks run in launch order). */
mmc_status mmc_serve_wait_buffer(mmc_server* server, int buffer);
mmc_status mmc_serve_destroy(mmc_server* server);

/* Relaxed device-scope atomicOr throughput over `words` u32 words at `buf`
 * (device, zeroed by the caller): iters per thread, random word per op.
 * returning != 0 uses the value (atom), else it is discarded (red).
 * contended != 0 makes every lane of a warp hit the same word. */
mmc_status mmc_atomic_peak(uint32_t* buf, uint64_t words, uint32_t blocks, uint32_t threads_per_block, uint32_t iters,
                           int returning, int contended, unsigned long long* sink, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MALLOCMC_GB300_H */

/* scatter_oracle.c — CPU restatement of mallocMC's Scatter heap (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY; see scatter_oracle.h for what it restates and
 * under which CPU-backend semantics. Each function names the reference lines
 * (paths relative to the mallocMC project root) it follows. All arithmetic is
 * uint32 where the reference's is, so wrap-around matches.
 *
 * Deliberate divergence (memory safety): the reference's second page-based
 * search (Scatter.hpp:834-836 -> :783-787) starts at index numpages and so
 * reads one PTE past the end of the PTE array (in the reference's layout that
 * is the first region counter). Here, as in the CUDA heap, a page index >=
 * numpages is treated as "in use". Every other behaviour is the reference's.
 */
#define _GNU_SOURCE
#include "scatter_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef struct
{
    uint32_t chunksize;
    uint32_t count;
    uint32_t bitmask;
} oc_pte; /* Scatter.hpp:213-230 (12 bytes, the reference's array-of-structs layout) */

struct oc_heap
{
    oc_config cfg;
    /* derived constants, Scatter.hpp:166-187 */
    uint32_t HierarchyThreshold;
    uint32_t minChunkSize;
    uint32_t maxOnPageMasks;
    /* heap header, Scatter.hpp:263-271 */
    uint8_t* pool;
    uint8_t* pages;
    oc_pte* ptes;
    uint32_t* regions;
    uint64_t memsize;
    uint32_t numpages;
    uint32_t numregions;
    uint32_t accessblocks;
    uint32_t pagebasedMutex;
    uint32_t firstFreePageBased;
    uint32_t firstfreeblock;
};

/* ---- atomics (alpaka::atomicOp on the CPU backends, sequentially consistent) ---- */
static inline uint32_t a_add(uint32_t* p, uint32_t v) { return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST); }
static inline uint32_t a_sub(uint32_t* p, uint32_t v) { return __atomic_fetch_sub(p, v, __ATOMIC_SEQ_CST); }
static inline uint32_t a_or(uint32_t* p, uint32_t v) { return __atomic_fetch_or(p, v, __ATOMIC_SEQ_CST); }
static inline uint32_t a_and(uint32_t* p, uint32_t v) { return __atomic_fetch_and(p, v, __ATOMIC_SEQ_CST); }
static inline uint32_t a_exch(uint32_t* p, uint32_t v) { return __atomic_exchange_n(p, v, __ATOMIC_SEQ_CST); }
static inline uint32_t a_cas(uint32_t* p, uint32_t cmp, uint32_t v)
{
    __atomic_compare_exchange_n(p, &cmp, v, 0, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
    return cmp; /* old value, as atomicCAS returns */
}
static inline uint32_t a_min(uint32_t* p, uint32_t v)
{
    uint32_t old = __atomic_load_n(p, __ATOMIC_SEQ_CST);
    while(!__atomic_compare_exchange_n(p, &old, old < v ? old : v, 1, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST))
        ;
    return old;
}
static inline uint32_t a_max(uint32_t* p, uint32_t v)
{
    uint32_t old = __atomic_load_n(p, __ATOMIC_SEQ_CST);
    while(!__atomic_compare_exchange_n(p, &old, old > v ? old : v, 1, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST))
        ;
    return old;
}
static inline uint32_t ld(const uint32_t* p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }
static inline void st(uint32_t* p, uint32_t v) { __atomic_store_n(p, v, __ATOMIC_RELAXED); }
static inline void fence_device(void) { __atomic_thread_fence(__ATOMIC_SEQ_CST); }

/* ---- intrinsics with CPU-backend semantics, mallocMC_utils.hpp:72-245 ---- */
#define OC_WARPSIZE 1u /* mallocMC_utils.hpp:85-87 */
static inline uint32_t laneid(void) { return 0u; } /* :99-101 */
static inline uint32_t warpid(void) { return 0u; } /* :121-123 */
static inline uint32_t smid(void) { return 0u; }   /* :134-136 */
static inline uint32_t ffs32(uint32_t m) { return m ? (uint32_t) __builtin_ctz(m) + 1u : 0u; } /* :205-222 */
static inline uint32_t popc32(uint32_t m) { return (uint32_t) __builtin_popcount(m); }           /* :224-245 */
static inline uint32_t umin(uint32_t a, uint32_t b) { return a < b ? a : b; }
static inline uint32_t umax(uint32_t a, uint32_t b) { return a > b ? a : b; }
static inline uint32_t divup(uint32_t a, uint32_t b) { return (a + b - 1u) / b; } /* mallocMC_utils.hpp:177-181 */

/* Shrink::applyPadding (Shrink.hpp:132-137), Noop::applyPadding (alignmentPolicies/Noop.hpp:55-59) */
static inline uint32_t apply_padding(const oc_heap* h, uint32_t bytes)
{
    uint32_t a = h->cfg.dataAlignment;
    if(a <= 1u)
        return bytes;
    uint32_t clear = a - 1u;
    return (bytes + clear) & ~clear;
}

static inline uint8_t* page_data(oc_heap* h, uint32_t page) { return h->pages + (uint64_t) page * h->cfg.pagesize; }

/* Page::init, Scatter.hpp:247-258: zero the last maxOnPageMasks words of a page */
static void page_init(oc_heap* h, uint32_t page)
{
    uint32_t* w = (uint32_t*) (page_data(h, page) + h->cfg.pagesize - 4u * h->maxOnPageMasks);
    for(uint32_t i = 0; i < h->maxOnPageMasks; ++i)
        st(&w[i], 0u);
}

/* randInit, Scatter.hpp:277-281 */
static inline uint32_t rand_init(void) { return laneid(); }

/* nextspot, Scatter.hpp:293-304 */
static inline uint32_t nextspot(uint32_t bitfield, uint32_t spot, uint32_t spots)
{
    const uint32_t low_part = (spot + 1u) == 32u ? 0u : (bitfield >> (spot + 1u));
    const uint32_t high_part = (bitfield << (spots - (spot + 1u)));
    const uint32_t selection_mask = spots == 32u ? ~0u : ((1u << spots) - 1u);
    bitfield = (high_part | low_part) & selection_mask;
    const uint32_t step = ffs32(~bitfield);
    return (spot + step) % spots;
}

/* onPageMasksPosition, Scatter.hpp:315-318 */
static inline uint32_t* on_page_masks(oc_heap* h, uint32_t page, uint32_t nMasks)
{
    return (uint32_t*) (page_data(h, page) + h->cfg.pagesize - 4u * nMasks);
}

/* usespot, Scatter.hpp:329-347 */
static int usespot(uint32_t* bitfield, uint32_t spots)
{
    uint32_t spot = rand_init() % spots;
    for(;;)
    {
        const uint32_t mask = 1u << spot;
        const uint32_t old = a_or(bitfield, mask);
        if((old & mask) == 0u)
            return (int) spot;
        if(popc32(old) >= spots)
            return -1;
        spot = nextspot(old, spot, spots);
    }
}

/* calcAdditionalChunks, Scatter.hpp:365-381. The (int) casts in the reference
 * collapse to unsigned arithmetic ((int)x * uint32 is uint32) and the
 * max(int 0, unsigned)/min(int 31, unsigned) compare as unsigned (CUDA ::max/::min). */
static inline uint32_t calc_additional_chunks(const oc_heap* h, uint32_t fullsegments, uint32_t segmentsize,
                                              uint32_t chunksize)
{
    if(fullsegments != 32u)
    {
        const uint32_t rest = h->cfg.pagesize - fullsegments * segmentsize - 4u;
        return umin(31u, umax(0u, rest) / chunksize);
    }
    return 0u;
}

/* addChunkHierarchy, Scatter.hpp:397-421 */
static void* add_chunk_hierarchy(oc_heap* h, uint32_t chunksize, uint32_t fullsegments, uint32_t additional_chunks,
                                 uint32_t page)
{
    const uint32_t segments = fullsegments + (additional_chunks > 0u ? 1u : 0u);
    uint32_t spot = rand_init() % segments;
    const uint32_t mask = ld(&h->ptes[page].bitmask);
    if((mask & (1u << spot)) != 0u)
        spot = nextspot(mask, spot, segments);
    const uint32_t tries = segments - popc32(mask);
    uint32_t* onpagemasks = on_page_masks(h, page, segments);
    for(uint32_t i = 0; i < tries; ++i)
    {
        const int hspot = usespot(&onpagemasks[spot], spot < fullsegments ? 32u : additional_chunks);
        if(hspot != -1)
            return page_data(h, page) + (32u * spot + (uint32_t) hspot) * chunksize;
        a_or(&h->ptes[page].bitmask, 1u << spot);
        spot = nextspot(mask, spot, segments);
    }
    return NULL;
}

/* addChunkNoHierarchy, Scatter.hpp:432-443 */
static void* add_chunk_no_hierarchy(oc_heap* h, uint32_t chunksize, uint32_t page, uint32_t spots)
{
    const int spot = usespot(&h->ptes[page].bitmask, spots);
    if(spot == -1)
        return NULL;
    return page_data(h, page) + (uint32_t) spot * chunksize;
}

/* tryUsePage, Scatter.hpp:454-518. [lo, hi] is isChunkSizeInRange. */
static void* try_use_page(oc_heap* h, uint32_t page, uint32_t chunksize, uint32_t lo, uint32_t hi)
{
    const uint32_t P = h->cfg.pagesize;
    void* chunk_ptr = NULL;
    const uint32_t filllevel = a_add(&h->ptes[page].count, 1u);
    int tryAllocMem = !h->cfg.resetfreedpages;
    if(h->cfg.resetfreedpages && filllevel < P)
    {
        const uint32_t oldChunksize = a_cas(&h->ptes[page].chunksize, 0u, chunksize);
        if(oldChunksize == 0u || (oldChunksize >= lo && oldChunksize <= hi))
            tryAllocMem = 1;
        if(oldChunksize != 0u)
            chunksize = oldChunksize;
    }
    if(tryAllocMem)
    {
        if(chunksize <= h->HierarchyThreshold)
        {
            const uint32_t segmentsize = chunksize * 32u + 4u;
            const uint32_t fullsegments = umin(32u, P / segmentsize);
            const uint32_t additional_chunks = calc_additional_chunks(h, fullsegments, segmentsize, chunksize);
            if(filllevel < fullsegments * 32u + additional_chunks)
                chunk_ptr = add_chunk_hierarchy(h, chunksize, fullsegments, additional_chunks, page);
        }
        else
        {
            const uint32_t chunksinpage = umin(P / chunksize, 32u);
            if(filllevel < chunksinpage)
                chunk_ptr = add_chunk_no_hierarchy(h, chunksize, page, chunksinpage);
        }
    }
    if(chunk_ptr == NULL)
        a_sub(&h->ptes[page].count, 1u);
    return chunk_ptr;
}

/* allocChunked, Scatter.hpp:527-637 */
static void* alloc_chunked(oc_heap* h, uint32_t bytes)
{
    const oc_config* c = &h->cfg;
    const uint32_t P = c->pagesize;
    const uint32_t R = c->regionsize;
    const uint32_t paddedMinChunkSize = apply_padding(h, h->minChunkSize);
    const uint32_t minAllocation = umax(bytes, paddedMinChunkSize);
    const uint32_t numpages = h->numpages;
    const uint32_t pagesperblock = numpages / h->accessblocks;
    const uint32_t reloff = OC_WARPSIZE * minAllocation / P;
    const uint32_t start_page_in_block
        = (minAllocation * c->hashingK + c->hashingDistMP * smid() + (c->hashingDistWP + c->hashingDistWPRel * reloff) * warpid())
        % pagesperblock;
    const uint32_t maxchunksize = umin(P, umax(c->wastefactor * bytes, paddedMinChunkSize));
    const uint32_t global_start_page = start_page_in_block + ld(&h->firstfreeblock) * pagesperblock;

    uint32_t checklevel = R * 3u / 4u;
    for(uint32_t finder = 0; finder < 2u; ++finder)
    {
        uint32_t global_page = global_start_page;
        do
        {
            const uint32_t region = global_page / R;
            const uint32_t regionfilllevel = ld(&h->regions[region]);
            const uint32_t region_offset = region * R;
            if(regionfilllevel < checklevel)
            {
                uint32_t page_in_region = global_page;
                do
                {
                    const uint32_t beforeChunkSize = a_cas(&h->ptes[page_in_region].chunksize, 0u, minAllocation);
                    uint32_t useChunkSize = 0u;
                    if(beforeChunkSize == 0u)
                        useChunkSize = minAllocation;
                    else if(beforeChunkSize >= bytes && beforeChunkSize <= maxchunksize)
                        useChunkSize = beforeChunkSize;
                    if(useChunkSize != 0u)
                    {
                        void* res = try_use_page(h, page_in_region, useChunkSize, bytes, maxchunksize);
                        if(res != NULL)
                            return res;
                    }
                    page_in_region = region_offset + ((page_in_region + 1u) % R);
                } while(page_in_region != global_page);

                if(regionfilllevel + 1u <= R)
                    a_cas(&h->regions[region], regionfilllevel, regionfilllevel + 1u);
            }
            global_page = (global_page + R) % numpages;
            if(global_page % pagesperblock == 0u)
            {
                const uint32_t access_block_id = global_page / pagesperblock;
                if(access_block_id > ld(&h->firstfreeblock))
                    st(&h->firstfreeblock, access_block_id);
            }
        } while(global_page != global_start_page);
        checklevel = R + 1u;
    }
    return NULL;
}

/* deallocChunked, Scatter.hpp:646-736 */
static void dealloc_chunked(oc_heap* h, void* mem, uint32_t page, uint32_t chunksize)
{
    const uint32_t P = h->cfg.pagesize;
    const uint32_t inpage_offset = (uint32_t) ((uint8_t*) mem - page_data(h, page));
    if(chunksize <= h->HierarchyThreshold)
    {
        const uint32_t segmentsize = chunksize * 32u + 4u;
        const uint32_t fullsegments = umin(32u, P / segmentsize);
        const uint32_t additional_chunks = calc_additional_chunks(h, fullsegments, segmentsize, chunksize);
        const uint32_t segment = inpage_offset / (chunksize * 32u);
        const uint32_t withinsegment = (inpage_offset - segment * (chunksize * 32u)) / chunksize;
        const uint32_t nMasks = fullsegments + (additional_chunks > 0u ? 1u : 0u);
        uint32_t* onpagemasks = on_page_masks(h, page, nMasks);
        a_and(&onpagemasks[segment], ~(1u << withinsegment));
        a_and(&h->ptes[page].bitmask, ~(1u << segment));
    }
    else
    {
        const uint32_t segment = inpage_offset / chunksize;
        a_and(&h->ptes[page].bitmask, ~(1u << segment));
    }

    uint32_t oldfilllevel = 0u;
    if(h->cfg.resetfreedpages)
    {
        oldfilllevel = a_cas(&h->ptes[page].count, 1u, P);
        if(oldfilllevel == 1u)
        {
            page_init(h, page);
            a_cas(&h->ptes[page].chunksize, chunksize, 0u);
            fence_device();
            a_sub(&h->ptes[page].count, P);
        }
        else
            oldfilllevel = a_sub(&h->ptes[page].count, 1u);
    }
    else
        oldfilllevel = a_sub(&h->ptes[page].count, 1u);

    if(oldfilllevel == P / 2u / chunksize)
    {
        const uint32_t region = page / h->cfg.regionsize;
        a_exch(&h->regions[region], 0u);
        const uint32_t pagesperblock = h->numpages / h->accessblocks;
        const uint32_t block = page / pagesperblock;
        if(warpid() + laneid() == 0u)
            a_min(&h->firstfreeblock, block);
    }
}

/* chunksize of a page for the page-based scan; index numpages (one past the
 * end, reached by the reference's second search) reads as "in use" here. */
static inline uint32_t scan_chunksize(oc_heap* h, uint32_t page)
{
    return page < h->numpages ? ld(&h->ptes[page].chunksize) : 1u;
}

/* markpages, Scatter.hpp:745-764 */
static int markpages(oc_heap* h, uint32_t startpage, uint32_t pages, uint32_t bytes)
{
    uint32_t abord = UINT32_MAX;
    for(uint32_t trypage = startpage; trypage < startpage + pages; ++trypage)
    {
        const uint32_t old = a_cas(&h->ptes[trypage].chunksize, 0u, bytes);
        if(old != 0u)
        {
            abord = trypage;
            break;
        }
    }
    if(abord == UINT32_MAX)
        return 1;
    for(uint32_t trypage = startpage; trypage < abord; ++trypage)
        a_cas(&h->ptes[trypage].chunksize, bytes, 0u);
    return 0;
}

/* allocPageBasedSingleRegion, Scatter.hpp:775-813 */
static void* alloc_page_based_single_region(oc_heap* h, uint32_t startpage, uint32_t endpage, uint32_t bytes)
{
    const uint32_t pagestoalloc = divup(bytes, h->cfg.pagesize);
    uint32_t freecount = 0;
    int left_free = 0;
    for(uint32_t search_page = startpage + 1u; search_page > endpage;)
    {
        --search_page;
        if(scan_chunksize(h, search_page) == 0u)
        {
            if(++freecount == pagestoalloc)
            {
                if(markpages(h, search_page, pagestoalloc, bytes))
                {
                    if(!left_free)
                    {
                        /* the reference stores search_page - 1, which wraps to
                         * 0xFFFFFFFF for a run ending at page 0 (Scatter.hpp:800-804) */
                        uint32_t nf = search_page - 1u;
                        if(!h->cfg.reference_quirks && search_page == 0u)
                            nf = 0u;
                        a_cas(&h->firstFreePageBased, startpage, nf);
                    }
                    return page_data(h, search_page);
                }
            }
        }
        else
        {
            left_free = 1;
            freecount = 0;
        }
    }
    return NULL;
}

/* allocPageBasedSingle, Scatter.hpp:824-840 */
static void* alloc_page_based_single(oc_heap* h, uint32_t bytes)
{
    while(a_exch(&h->pagebasedMutex, 1u) != 0u)
        ;
    const uint32_t spage = ld(&h->firstFreePageBased);
    void* res = alloc_page_based_single_region(h, spage, 0u, bytes);
    if(res == NULL)
        res = alloc_page_based_single_region(h, h->numpages, spage, bytes);
    a_exch(&h->pagebasedMutex, 0u);
    return res;
}

/* deallocPageBased, Scatter.hpp:874-886 */
static void dealloc_page_based(oc_heap* h, uint32_t page, uint32_t bytes)
{
    const uint32_t pages = divup(bytes, h->cfg.pagesize);
    for(uint32_t p = page; p < page + pages; ++p)
        page_init(h, p);
    fence_device();
    for(uint32_t p = page; p < page + pages; ++p)
        a_cas(&h->ptes[p].chunksize, bytes, 0u);
    a_max(&h->firstFreePageBased, page + pages - 1u);
}

/* create, Scatter.hpp:895-912 (allocPageBased's lane serialisation, :848-866, is a
 * single call with one lane) */
static void* create(oc_heap* h, uint32_t bytes)
{
    if(bytes == 0u)
        return NULL;
    if(bytes <= h->cfg.pagesize)
        return alloc_chunked(h, bytes);
    return alloc_page_based_single(h, bytes);
}

/* destroy, Scatter.hpp:918-946 */
static void destroy(oc_heap* h, void* mem)
{
    if(mem == NULL)
        return;
    const uint32_t P = h->cfg.pagesize;
    const uint32_t page = (uint32_t) (((uint8_t*) mem - h->pages) / P);
    const uint32_t chunksize = ld(&h->ptes[page].chunksize);
    if(chunksize == 0u)
        return; /* the reference divides by zero here (freeing a pointer of an unformatted page) */
    const uint32_t inpage_offset = (uint32_t) ((uint8_t*) mem - page_data(h, page));
    const uint32_t block = inpage_offset / chunksize;
    const uint32_t inblockoffset = inpage_offset - block * chunksize;
    if(inblockoffset != 0u)
    {
        uint32_t* counter = (uint32_t*) (page_data(h, page) + block * chunksize);
        const uint32_t old = a_sub(counter, 1u);
        if(old != 1u)
            return;
        mem = (void*) counter;
    }
    if(chunksize < P || (!h->cfg.reference_quirks && chunksize == P))
        dealloc_chunked(h, mem, page, chunksize);
    else
        dealloc_page_based(h, page, chunksize);
}

/* DeviceAllocator::malloc, device_allocator.hpp:72-82: pad (size_t -> uint32
 * narrowing, Shrink.hpp:133), collect/distribute are the identity with one
 * lane, ReturnNull turns a failure into NULL. */
void* oc_malloc(oc_heap* h, uint64_t bytes)
{
    const uint32_t req = apply_padding(h, (uint32_t) bytes);
    void* p = create(h, req);
    return p; /* isOOM -> ReturnNull::handleOOM returns nullptr == p */
}

void oc_free(oc_heap* h, void* p) { destroy(h, p); }

/* countFreeChunksInPage, Scatter.hpp:1112-1139 */
static uint32_t count_free_chunks_in_page(oc_heap* h, uint32_t page, uint32_t chunksize)
{
    const uint32_t P = h->cfg.pagesize;
    const uint32_t filledChunks = ld(&h->ptes[page].count);
    if(chunksize <= h->HierarchyThreshold)
    {
        const uint32_t segmentsize = chunksize * 32u + 4u;
        const uint32_t fullsegments = umin(32u, P / segmentsize);
        const uint32_t additional_chunks = calc_additional_chunks(h, fullsegments, segmentsize, chunksize);
        const uint32_t level2Chunks = fullsegments * 32u + additional_chunks;
        return level2Chunks - filledChunks;
    }
    const uint32_t chunksinpage = umin(P / chunksize, 32u);
    return chunksinpage - filledChunks;
}

/* getAvailaibleSlotsDeviceFunction, Scatter.hpp:1158-1219 */
static uint32_t slots_device_function(oc_heap* h, uint64_t slotSize, uint32_t gid, uint32_t stride)
{
    const uint32_t P = h->cfg.pagesize;
    uint32_t slotcount = 0;
    if(slotSize < P)
    {
        for(uint32_t currentpage = gid; currentpage < h->numpages; currentpage += stride)
        {
            const uint32_t maxchunksize = umin(P, h->cfg.wastefactor * (uint32_t) slotSize);
            uint32_t chunksize = ld(&h->ptes[currentpage].chunksize);
            if((uint64_t) chunksize >= slotSize && chunksize <= maxchunksize)
                slotcount += count_free_chunks_in_page(h, currentpage, chunksize);
            else if(chunksize == 0u)
            {
                chunksize = umax((uint32_t) slotSize, apply_padding(h, h->minChunkSize));
                slotcount += count_free_chunks_in_page(h, currentpage, chunksize);
            }
        }
    }
    else
    {
        if(gid > 0u)
            return 0u;
        const uint32_t pagestoalloc = divup((uint32_t) slotSize, P);
        uint32_t freecount = 0;
        for(uint32_t currentpage = h->numpages; currentpage > 0u;)
        {
            --currentpage;
            if(ld(&h->ptes[currentpage].chunksize) == 0u)
            {
                if(++freecount == pagestoalloc)
                {
                    freecount = 0;
                    ++slotcount;
                }
            }
            else
                freecount = 0;
        }
    }
    return slotcount;
}

/* getAvailableSlotsHost, Scatter.hpp:1235-1295: 64 blocks x min(256, maxThreads)
 * threads; on the CPU-serial backend that is 64 workers of one thread. The sum
 * is order-independent modulo 2^32. Padding first: allocator.hpp:230. */
uint32_t oc_available_slots(oc_heap* h, uint64_t slotSize)
{
    slotSize = apply_padding(h, (uint32_t) slotSize);
    uint32_t total = 0;
    for(uint32_t gid = 0; gid < 64u; ++gid)
        total += slots_device_function(h, slotSize, gid, 64u);
    return total;
}

/* getAvailableSlotsAccelerator, Scatter.hpp:1311-1352, one active thread;
 * padding first: device_allocator.hpp:103. */
uint32_t oc_available_slots_accelerator(oc_heap* h, uint64_t slotSize)
{
    slotSize = apply_padding(h, (uint32_t) slotSize);
    if(slotSize == 0u)
        return 0u;
    return slots_device_function(h, slotSize, 0u, 1u);
}

/* Allocator::alloc + initDeviceFunction, allocator.hpp:136-159, Scatter.hpp:956-1049 */
int oc_heap_create(const oc_config* cfg, uint64_t memsize, oc_heap** out)
{
    *out = NULL;
    const uint32_t P = cfg->pagesize;
    if(P < 128u || cfg->regionsize == 0u || cfg->accessblocksize == 0u)
        return OC_ERR_CONFIG;
    oc_heap* h = (oc_heap*) calloc(1, sizeof(oc_heap));
    if(!h)
        return OC_ERR_NOMEM;
    h->cfg = *cfg;
    /* Scatter.hpp:166-187 (sizeof(uint32) = 4) */
    h->HierarchyThreshold = (P - 2u * 4u) / 33u;
    h->minChunkSize = (P - 32u * 4u) / (32u * 32u);
    const uint32_t minSegmentSize = 32u * h->minChunkSize + 4u;
    const uint32_t onPageMasks
        = h->minChunkSize > h->HierarchyThreshold ? 0u : (P + (minSegmentSize - 1u)) / minSegmentSize;
    h->maxOnPageMasks = umin(32u, onPageMasks);

    /* the reference's pool: AlpakaBuf on the CPU backend, 16-byte aligned or
     * better, so Shrink::alignPool (Shrink.hpp:109-130) changes nothing */
    h->pool = (uint8_t*) aligned_alloc(4096, (memsize + 4095u) & ~(uint64_t) 4095u);
    if(!h->pool)
    {
        free(h);
        return OC_ERR_NOMEM;
    }
    const uint32_t R = cfg->regionsize;
    uint32_t numregions = (uint32_t) (memsize / ((uint64_t) R * (sizeof(oc_pte) + P) + 4u));
    uint32_t numpages = numregions * R;
    const uint64_t memorysize = (uint64_t) numpages * P;
    const uint64_t numblocks = memorysize / cfg->accessblocksize;
    if(numblocks == 0u)
    {
        /* the reference divides by zero here (Scatter.hpp:993) */
        free(h->pool);
        free(h);
        return OC_ERR_CONFIG;
    }
    const uint64_t memoryperblock = memorysize / numblocks;
    const uint64_t pagesperblock = memoryperblock / P;
    const uint64_t regionsperblock = pagesperblock / R;
    numregions = (uint32_t) (numblocks * regionsperblock);
    numpages = numregions * R;
    if(numpages == 0u)
    {
        free(h->pool);
        free(h);
        return OC_ERR_CONFIG;
    }
    uint8_t* page = h->pool;
    oc_pte* ptes = (oc_pte*) (page + (uint64_t) numpages * P);
    uint32_t* regions = (uint32_t*) (ptes + numpages);
    if((uint8_t*) (regions + numregions) > h->pool + memsize)
    {
        --numregions;
        numpages = umin(numregions * R, numpages);
    }
    ptes = (oc_pte*) (page + (uint64_t) numpages * P);
    regions = (uint32_t*) (ptes + numpages);
    h->pages = page;
    h->ptes = ptes;
    h->regions = regions;
    h->memsize = memsize;
    h->numpages = numpages;
    h->numregions = numregions;
    h->accessblocks = (uint32_t) numblocks;
    for(uint32_t i = 0; i < numpages; ++i)
    {
        ptes[i].chunksize = ptes[i].count = ptes[i].bitmask = 0u;
        page_init(h, i);
    }
    for(uint32_t i = 0; i < numregions; ++i)
        regions[i] = 0u;
    h->firstfreeblock = 0u;
    h->pagebasedMutex = 0u;
    h->firstFreePageBased = numpages - 1u;
    *out = h;
    return OC_OK;
}

void oc_heap_destroy(oc_heap* h)
{
    if(!h)
        return;
    free(h->pool);
    free(h);
}

uint8_t* oc_pool(oc_heap* h) { return h->pool; }
uint32_t oc_numpages(oc_heap* h) { return h->numpages; }
uint32_t oc_accessblocks(oc_heap* h) { return h->accessblocks; }
uint32_t oc_numregions(oc_heap* h) { return h->numregions; }
uint32_t oc_max_on_page_masks(oc_heap* h) { return h->maxOnPageMasks; }
uint32_t oc_hierarchy_threshold(oc_heap* h) { return h->HierarchyThreshold; }

void oc_header(oc_heap* h, uint32_t out[3])
{
    out[0] = h->firstFreePageBased;
    out[1] = h->firstfreeblock;
    out[2] = h->pagebasedMutex;
}

void oc_snapshot_ptes(oc_heap* h, uint32_t* out3)
{
    for(uint32_t i = 0; i < h->numpages; ++i)
    {
        out3[3u * i + 0u] = h->ptes[i].chunksize;
        out3[3u * i + 1u] = h->ptes[i].count;
        out3[3u * i + 2u] = h->ptes[i].bitmask;
    }
}

void oc_snapshot_regions(oc_heap* h, uint32_t* out) { memcpy(out, h->regions, 4u * (size_t) h->numregions); }

void oc_snapshot_masks(oc_heap* h, uint32_t* out)
{
    const uint32_t n = h->maxOnPageMasks;
    for(uint32_t i = 0; i < h->numpages; ++i)
        memcpy(out + (size_t) i * n, page_data(h, i) + h->cfg.pagesize - 4u * n, 4u * (size_t) n);
}

void oc_load_state(oc_heap* h, const uint32_t* ptes3, const uint32_t* regions, const uint32_t* masks)
{
    const uint32_t n = h->maxOnPageMasks;
    for(uint32_t i = 0; i < h->numpages; ++i)
    {
        h->ptes[i].chunksize = ptes3[3u * i + 0u];
        h->ptes[i].count = ptes3[3u * i + 1u];
        h->ptes[i].bitmask = ptes3[3u * i + 2u];
        if(masks)
            memcpy(page_data(h, i) + h->cfg.pagesize - 4u * n, masks + (size_t) i * n, 4u * (size_t) n);
    }
    if(regions)
        memcpy(h->regions, regions, 4u * (size_t) h->numregions);
}

void oc_run_program(oc_heap* h, const uint8_t* kinds, const uint64_t* args, int64_t n, int64_t* out)
{
    for(int64_t i = 0; i < n; ++i)
    {
        out[i] = 0;
        switch(kinds[i])
        {
        case 'm':
        {
            void* p = oc_malloc(h, args[i]);
            out[i] = p ? (int64_t) ((uint8_t*) p - h->pool) : -1;
            break;
        }
        case 'f':
        {
            const int64_t j = (int64_t) args[i];
            if(j >= 0 && j < i && kinds[j] == 'm' && out[j] >= 0)
                oc_free(h, h->pool + out[j]);
            break;
        }
        case 's': out[i] = oc_available_slots(h, args[i]); break;
        case 'd': out[i] = oc_available_slots_accelerator(h, args[i]); break;
        default: break;
        }
    }
}

uint64_t oc_mix64(uint64_t seed, uint64_t a, uint64_t b)
{
    uint64_t z = seed + a * 0x9E3779B97F4A7C15ull + b * 0xD1B54A32D192ED03ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint32_t oc_frag_size(uint64_t seed, uint64_t i, uint32_t small_lo, uint32_t small_hi, uint32_t large_lo,
                      uint32_t large_hi, uint32_t large_permille)
{
    const uint64_t m = oc_mix64(seed, i, 0xF4A6ull);
    if((uint32_t) (m % 1000u) < large_permille)
    {
        /* log-uniform: exp2 of a uniform exponent, from 24 bits of the draw */
        const double u = (double) ((m >> 20) & 0xFFFFFFull) / 16777216.0;
        const double lo = (double) large_lo, hi = (double) large_hi;
        double v = lo * __builtin_exp(u * __builtin_log(hi / lo));
        uint32_t s = (uint32_t) v;
        return s < large_lo ? large_lo : (s > large_hi ? large_hi : s);
    }
    return small_lo + (uint32_t) ((m >> 32) % (uint64_t) (small_hi - small_lo + 1u));
}

void oc_run_fragmentation(oc_heap* h, uint64_t seed, uint32_t small_lo, uint32_t small_hi, uint32_t large_lo,
                          uint32_t large_hi, uint32_t large_permille, uint64_t* out)
{
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    size_t cap = 1u << 20, n = 0;
    void** ptr = (void**) malloc(cap * sizeof(void*));
    uint32_t* sz = (uint32_t*) malloc(cap * sizeof(uint32_t));
    uint64_t i = 0, live = 0;
    for(;; ++i)
    {
        const uint32_t s = oc_frag_size(seed, i, small_lo, small_hi, large_lo, large_hi, large_permille);
        void* p = oc_malloc(h, s);
        if(!p)
            break;
        if(n == cap)
        {
            cap *= 2;
            ptr = (void**) realloc(ptr, cap * sizeof(void*));
            sz = (uint32_t*) realloc(sz, cap * sizeof(uint32_t));
        }
        ptr[n] = p;
        sz[n] = s;
        ++n;
        live += s;
    }
    out[0] = n;
    out[1] = live;
    /* seeded Fisher-Yates over the live list; free the first half */
    for(size_t k = n; k > 1; --k)
    {
        const size_t j = (size_t) (oc_mix64(seed, k, 0x5A11ull) % k);
        void* tp = ptr[k - 1];
        ptr[k - 1] = ptr[j];
        ptr[j] = tp;
        uint32_t ts = sz[k - 1];
        sz[k - 1] = sz[j];
        sz[j] = ts;
    }
    const size_t half = n / 2;
    for(size_t k = 0; k < half; ++k)
    {
        oc_free(h, ptr[k]);
        live -= sz[k];
    }
    out[2] = half;
    uint64_t n2 = 0;
    for(++i;; ++i)
    {
        const uint32_t s = oc_frag_size(seed, i, small_lo, small_hi, large_lo, large_hi, large_permille);
        void* p = oc_malloc(h, s);
        if(!p)
            break;
        ++n2;
        live += s;
    }
    out[3] = n2;
    out[4] = live;
    clock_gettime(CLOCK_MONOTONIC, &t1);
    out[5] = (uint64_t) (1e6 * ((double) (t1.tv_sec - t0.tv_sec) + 1e-9 * (double) (t1.tv_nsec - t0.tv_nsec)));
    free(ptr);
    free(sz);
}

/* ---- multi-threaded stress (the CPU baseline) ---- */
typedef struct
{
    oc_heap* h;
    uint64_t vthreads;
    uint32_t rounds, lo, hi, step;
    uint64_t seed;
    uint64_t next; /* shared virtual-thread counter */
    uint64_t pairs, nulls, bad;
} stress_ctx;

static void* stress_worker(void* arg)
{
    stress_ctx* s = (stress_ctx*) arg;
    const uint32_t nsizes = (s->hi - s->lo) / s->step + 1u;
    uint64_t pairs = 0, nulls = 0, bad = 0;
    for(;;)
    {
        const uint64_t t = __atomic_fetch_add(&s->next, 1u, __ATOMIC_RELAXED);
        if(t >= s->vthreads)
            break;
        for(uint32_t r = 0; r < s->rounds; ++r)
        {
            const uint64_t m = oc_mix64(s->seed, t, r);
            const uint32_t bytes = s->lo + ((uint32_t) (m >> 32) % nsizes) * s->step;
            uint64_t* p = (uint64_t*) oc_malloc(s->h, bytes);
            if(!p)
            {
                ++nulls;
                continue;
            }
            const uint32_t words = bytes / 8u;
            for(uint32_t i = 0; i < words; ++i)
                p[i] = m + i;
            for(uint32_t i = 0; i < words; ++i)
                bad += (p[i] != m + i);
            oc_free(s->h, p);
            ++pairs;
        }
    }
    __atomic_fetch_add(&s->pairs, pairs, __ATOMIC_RELAXED);
    __atomic_fetch_add(&s->nulls, nulls, __ATOMIC_RELAXED);
    __atomic_fetch_add(&s->bad, bad, __ATOMIC_RELAXED);
    return NULL;
}

uint64_t oc_run_stress(oc_heap* h, uint64_t vthreads, uint32_t rounds, uint64_t seed, uint32_t lo, uint32_t hi,
                       uint32_t step, int workers, uint64_t* nulls, uint64_t* bad, double* seconds)
{
    stress_ctx s;
    memset(&s, 0, sizeof(s));
    s.h = h;
    s.vthreads = vthreads;
    s.rounds = rounds;
    s.lo = lo;
    s.hi = hi;
    s.step = step ? step : 16u;
    s.seed = seed;
    if(workers < 1)
        workers = 1;
    pthread_t* th = (pthread_t*) calloc((size_t) workers, sizeof(pthread_t));
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for(int i = 1; i < workers; ++i)
        pthread_create(&th[i], NULL, stress_worker, &s);
    stress_worker(&s);
    for(int i = 1; i < workers; ++i)
        pthread_join(th[i], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    free(th);
    if(nulls)
        *nulls = s.nulls;
    if(bad)
        *bad = s.bad;
    if(seconds)
        *seconds = (double) (t1.tv_sec - t0.tv_sec) + 1e-9 * (double) (t1.tv_nsec - t0.tv_nsec);
    return s.pairs;
}

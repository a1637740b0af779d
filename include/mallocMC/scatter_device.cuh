/* scatter_device.cuh — device side of the GB300 ScatterAlloc heap.
 *
 * Header-only __device__ code: user kernels include it (directly or through
 * <mallocMC/mallocMC.hpp>) and call malloc/free/getAvailableSlots inline, as
 * with the reference's AllocatorHandleImpl (mallocMC_allocator_handle.hpp:35-63).
 * The algorithm is the reference's ScatterAlloc
 * (src/include/mallocMC/creationPolicies/Scatter.hpp); every function cites the
 * lines it follows. What is GB300-specific:
 *   - the handle carries every immutable heap field by value (kernel parameter
 *     space), so only the mutable words are read from memory;
 *   - the page-table entries are three word arrays (chunksize[], count[],
 *     bitmask[]) instead of an array of 12-byte structs: same bytes, same
 *     numpages, but scans read only the words they need, fully coalesced;
 *   - relaxed device-scope atomics (atom/red .relaxed.gpu) on L2-resident words
 *     and ld.relaxed.gpu for the racy metadata reads;
 *   - XMallocSIMD's warp coalescing uses __ballot_sync/__shfl_sync over the
 *     lanes that are active at the call, not shared-memory counters;
 *   - every spin is bounded: the page-based mutex gives up after a fixed
 *     number of backed-off tries, records MMC_DEVERR_TIMEOUT and returns NULL;
 *     the bit-claim retry loop gives up after MMC_USESPOT_MAX_TRIES.
 * Thread-id sources are a template parameter: GpuIds reads %laneid/%warpid/
 * %smid (mallocMC_utils.hpp:91-150); SerialIds is the reference CPU backend
 * (all zero, warp size 1), which makes one device thread reproduce the
 * reference's CPU-serial allocation sequence bit for bit.
 */
#pragma once

#include "../mallocmc_gb300.h"

#include <cstdint>

#ifndef MMC_USESPOT_MAX_TRIES
#define MMC_USESPOT_MAX_TRIES 256u
#endif
#ifndef MMC_MUTEX_MAX_SPINS
#define MMC_MUTEX_MAX_SPINS (1u << 22)
#endif

/* Mutable heap words, each on its own 128-byte line. */
struct mmc_heap_state
{
    uint32_t pagebasedMutex; /* Scatter.hpp:269 */
    uint32_t pad0[31];
    uint32_t firstFreePageBased; /* Scatter.hpp:270 */
    uint32_t pad1[31];
    uint32_t firstfreeblock; /* Scatter.hpp:271 */
    uint32_t pad2[31];
    uint32_t error_flags; /* MMC_DEVERR_* */
    uint32_t pad3[31];
    /* event counters, maintained only in builds with MMC_DEVICE_STATS (MMC_STAT_*) */
    unsigned long long stats[16];
};

#ifdef MMC_DEVICE_STATS
#define MMC_STAT(h, i) atomicAdd(&(h).state->stats[(i)], 1ull)
#define MMC_STAT_ADD(h, i, n) atomicAdd(&(h).state->stats[(i)], static_cast<unsigned long long>(n))
#else
#define MMC_STAT(h, i) ((void) 0)
#define MMC_STAT_ADD(h, i, n) ((void) 0)
#endif

namespace mmc
{
    namespace dev
    {
        using u32 = uint32_t;
        using u64 = uint64_t;

        /* ---------------------------------------------------------- thread ids */
        struct GpuIds
        {
            static constexpr u32 warpSize = 32u; /* mallocMC_utils.hpp:72-73 */
            static constexpr bool coalesce = true;
            /* read the racy first-free-block hint through L1 (it changes rarely
             * and a stale value only moves where the search starts) */
            static constexpr bool cachedHints = true;
            /* requests above a page take the multi-page path (SmallRequests
             * leaves it out) */
            static constexpr bool pageBased = true;
            __device__ static __forceinline__ u32 laneid()
            {
                u32 r;
                asm volatile("mov.u32 %0, %%laneid;" : "=r"(r));
                return r;
            }
            __device__ static __forceinline__ u32 warpid()
            {
                u32 r;
                asm volatile("mov.u32 %0, %%warpid;" : "=r"(r));
                return r;
            }
            __device__ static __forceinline__ u32 smid()
            {
                u32 r;
                asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
                return r;
            }
            /* the heap's policy values, read from the handle at run time */
            __device__ static __forceinline__ u32 reset(const mmc_device_handle& h) { return h.resetfreedpages; }
            __device__ static __forceinline__ u32 distribution(const mmc_device_handle& h) { return h.distribution; }
            __device__ static __forceinline__ u32 oom(const mmc_device_handle& h) { return h.oom_policy; }
            __device__ static __forceinline__ u32 alignment(const mmc_device_handle& h) { return h.dataAlignment; }
        };

        /* GpuIds with the policy values fixed at compile time, as the
         * reference's template parameters fix them (Scatter's resetfreedpages,
         * the distribution, OOM and alignment policies): code for the other
         * values drops out of the kernel, which shortens the malloc and free
         * paths the instruction cache holds (ncu counts instruction-fetch
         * stalls as the stress and batched kernels' top stall; 6 % and 11 %
         * faster measured). Only for heaps whose handle holds the same values
         * (matches()): the C++ Allocator picks it from its policies, the
         * library's kernels dispatch on matches(). */
        template<u32 RESET, u32 DIST, u32 OOM, u32 ALIGN>
        struct GpuIdsFixed : GpuIds
        {
            __device__ static __forceinline__ u32 reset(const mmc_device_handle&) { return RESET; }
            __device__ static __forceinline__ u32 distribution(const mmc_device_handle&) { return DIST; }
            __device__ static __forceinline__ u32 oom(const mmc_device_handle&) { return OOM; }
            __device__ static __forceinline__ u32 alignment(const mmc_device_handle&) { return ALIGN; }
            __host__ __device__ static bool matches(const mmc_device_handle& h)
            {
                return (h.resetfreedpages != 0u) == (RESET != 0u) && h.distribution == DIST && h.oom_policy == OOM
                       && (h.dataAlignment > 1u ? h.dataAlignment : 1u) == (ALIGN > 1u ? ALIGN : 1u);
            }
        };

        /* The configuration the bench's workloads and the reference's defaults
         * use: no page reset, XMallocSIMD, ReturnNull, Shrink<16>. */
        using GpuIdsDefault = GpuIdsFixed<0u, MMC_DIST_XMALLOCSIMD, MMC_OOM_RETURNNULL, 16u>;

        /* Base for a kernel whose requests never exceed a page after padding
         * (its caller knows the largest one): the multi-page search is left
         * out of it. That search is out-of-line code, and ptxas fits the
         * registers of every kernel that can call it around the search's own,
         * so a change in the search moved the chunk paths' register
         * allocation: the uniform stress kernel, which never asks for more
         * than 1 KiB, ran 2 to 17 % slower after changes to the search alone.
         * A request above a page in such a kernel returns NULL and sets
         * MMC_DEVERR_PAGEBASED. Frees are unchanged. */
        template<class Base>
        struct SmallRequests : Base
        {
            static constexpr bool pageBased = false;
        };

        /* The reference's CPU-backend semantics (mallocMC_utils.hpp:85-87, 99-101, 121-123, 134-136). */
        struct SerialIds
        {
            static constexpr u32 warpSize = 1u;
            static constexpr bool coalesce = false; /* XMallocSIMD.hpp:136-137 */
            static constexpr bool cachedHints = false;
            static constexpr bool pageBased = true;
            __device__ static __forceinline__ u32 laneid() { return 0u; }
            __device__ static __forceinline__ u32 warpid() { return 0u; }
            __device__ static __forceinline__ u32 smid() { return 0u; }
            __device__ static __forceinline__ u32 reset(const mmc_device_handle& h) { return h.resetfreedpages; }
            __device__ static __forceinline__ u32 distribution(const mmc_device_handle& h) { return h.distribution; }
            __device__ static __forceinline__ u32 oom(const mmc_device_handle& h) { return h.oom_policy; }
            __device__ static __forceinline__ u32 alignment(const mmc_device_handle& h) { return h.dataAlignment; }
        };

        /* ---------------------------------------------------- memory helpers */
        __device__ __forceinline__ u32 ld_rlx(const u32* p)
        {
            u32 v;
            asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
            return v;
        }
        __device__ __forceinline__ uint4 ld_rlx_v4(const u32* p)
        {
            uint4 v;
            asm volatile("ld.relaxed.gpu.global.v4.u32 {%0, %1, %2, %3}, [%4];"
                         : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                         : "l"(p)
                         : "memory");
            return v;
        }
        __device__ __forceinline__ void st_rlx(u32* p, u32 v)
        {
            asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
        }
        /* fence.release.gpu: this thread's earlier memory operations are
         * performed before its later writes and atomics, for every thread of
         * the GPU. (It measured 6 % faster on the uniform stress than
         * fence.acq_rel.gpu, which also orders the later reads; the free
         * needs only the release.) */
        __device__ __forceinline__ void release_fence() { asm volatile("fence.release.gpu;" ::: "memory"); }
        __device__ __forceinline__ u32 lanemask_lt()
        {
            u32 r;
            asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
            return r;
        }
        __device__ __forceinline__ u32 umin(u32 a, u32 b) { return a < b ? a : b; }
        __device__ __forceinline__ u32 umax(u32 a, u32 b) { return a > b ? a : b; }
        __device__ __forceinline__ u32 divup(u32 a, u32 b) { return (a + b - 1u) / b; }

        /* Shrink::applyPadding (Shrink.hpp:132-137) / Noop (alignmentPolicies/Noop.hpp:55-59). */
        __host__ __device__ __forceinline__ u32 apply_padding(u32 align, u32 bytes)
        {
            if(align <= 1u)
                return bytes;
            const u32 clear = align - 1u;
            return (bytes + clear) & ~clear;
        }

        __device__ __forceinline__ char* page_data(const mmc_device_handle& h, u32 page)
        {
            return h.pages + static_cast<u64>(page) * h.pagesize;
        }

        /* onPageMasksPosition, Scatter.hpp:315-318 */
        __device__ __forceinline__ u32* on_page_masks(const mmc_device_handle& h, u32 page, u32 nMasks)
        {
            return reinterpret_cast<u32*>(page_data(h, page) + h.pagesize - 4u * nMasks);
        }

        /* Page::init, Scatter.hpp:247-258: zero the words that can hold on-page masks. */
        __device__ __forceinline__ void page_init(const mmc_device_handle& h, u32 page)
        {
            u32* w = on_page_masks(h, page, h.maxOnPageMasks);
            for(u32 i = 0; i < h.maxOnPageMasks; ++i)
                st_rlx(w + i, 0u);
        }

        __device__ __forceinline__ void set_error(const mmc_device_handle& h, u32 bits)
        {
            atomicOr(&h.state->error_flags, bits);
        }

        /* ------------------------------------------------ free-page bitmap
         * h.freemap has one bit per page, set while the page's chunk size is
         * 0; the concurrent multi-page search reads it instead of the chunk
         * sizes, 32 pages per word (no counterpart in the reference, which
         * scans the page table). The chunk size stays the authority: a run is
         * owned only once markpages' CASes succeed, so a bit set on a used
         * page costs the search a failed CAS, as a lost run does. What must
         * not happen is a clear bit on a free page for longer than a free is
         * in flight, or the search would skip free pages. So: every change of
         * a chunk size to 0 (a free, a page reset, a markpages roll-back) sets
         * the bit after its CAS; every change from 0 clears the bit either
         * before its CAS, or after it while nothing can free the page yet
         * (markpages' run before it is handed out; a reset-mode format while
         * the caller holds a fill slot), and a fence then waits for the clear
         * to be performed, so no clear can land after a later free's set. */
        __device__ __forceinline__ void freemap_clear_acked(u32* fm, u32 page)
        {
            atomicAnd(&fm[page >> 5], ~(1u << (page & 31u)));
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
        }

        __device__ __forceinline__ void freemap_set(u32* fm, u32 page)
        {
            atomicOr(&fm[page >> 5], 1u << (page & 31u));
        }

        /* set (free) or clear the bits of pages [first, first + n), one atomic per word */
        __device__ inline void freemap_range(u32* fm, u32 first, u32 n, bool free)
        {
            for(u32 p = first, end = first + n; p < end;)
            {
                const u32 b = p & 31u;
                const u32 cnt = umin(32u - b, end - p);
                const u32 mask = cnt == 32u ? 0xFFFFFFFFu : ((1u << cnt) - 1u) << b;
                if(free)
                    atomicOr(&fm[p >> 5], mask);
                else
                    atomicAnd(&fm[p >> 5], ~mask);
                p += cnt;
            }
        }

        /* nextspot, Scatter.hpp:293-304 */
        __device__ __forceinline__ u32 nextspot(u32 bitfield, u32 spot, u32 spots)
        {
            const u32 low_part = (spot + 1u) == 32u ? 0u : (bitfield >> (spot + 1u));
            const u32 high_part = (bitfield << (spots - (spot + 1u)));
            const u32 selection_mask = spots == 32u ? ~0u : ((1u << spots) - 1u);
            bitfield = (high_part | low_part) & selection_mask;
            const u32 step = static_cast<u32>(__ffs(static_cast<int>(~bitfield)));
            return (spot + step) % spots;
        }

        /* usespot's retry sequence (Scatter.hpp:334-346) after an atomicOr at
         * `spot` returned `old` with that bit already set: stop when the word is
         * full, else try the next free spot of the returned word. Bounded by
         * MMC_USESPOT_MAX_TRIES lost races, after which the word counts as full,
         * which every caller already handles. */
        __device__ __forceinline__ int usespot_continue(u32* bitfield, u32 spots, u32 spot, u32 old)
        {
            for(u32 it = 1; it < MMC_USESPOT_MAX_TRIES; ++it)
            {
                if(static_cast<u32>(__popc(old)) >= spots)
                    return -1;
                spot = nextspot(old, spot, spots);
                const u32 mask = 1u << spot;
                old = atomicOr(bitfield, mask);
                if((old & mask) == 0u)
                    return static_cast<int>(spot);
            }
            return -1;
        }

        /* usespot, Scatter.hpp:329-347 (first spot laneid % spots, randInit :277-281) */
        template<class Ids>
        __device__ __forceinline__ int usespot(u32* bitfield, u32 spots)
        {
            const u32 spot = Ids::laneid() % spots;
            const u32 mask = 1u << spot;
            const u32 old = atomicOr(bitfield, mask);
            if((old & mask) == 0u)
                return static_cast<int>(spot);
            return usespot_continue(bitfield, spots, spot, old);
        }

        /* calcAdditionalChunks, Scatter.hpp:365-381: the (int) casts collapse to
         * unsigned arithmetic and CUDA's ::max/::min(int, unsigned) compare unsigned. */
        __device__ __forceinline__ u32 calc_additional_chunks(u32 pagesize, u32 fullsegments, u32 segmentsize,
                                                              u32 chunksize)
        {
            if(fullsegments != 32u)
                return umin(31u, (pagesize - fullsegments * segmentsize - 4u) / chunksize);
            return 0u;
        }

        /* Geometry of a page formatted with a chunk size (tryUsePage :493-508,
         * deallocChunked :652-660, countFreeChunksInPage :1116-1138). */
        struct ChunkGeom
        {
            bool hier;        /* chunksize <= HierarchyThreshold: on-page segment masks */
            u32 fullsegments; /* hierarchical: segments of 32 chunks */
            u32 additional;   /* hierarchical: chunks in the last, partial segment */
            u32 segments;     /* hierarchical: on-page mask words */
            u32 capacity;     /* chunks the page holds */
        };

        __device__ __forceinline__ ChunkGeom chunk_geom(const mmc_device_handle& h, u32 chunksize)
        {
            ChunkGeom g;
            g.hier = chunksize <= h.hierarchyThreshold;
            if(g.hier)
            {
                const u32 segmentsize = chunksize * 32u + 4u;
                g.fullsegments = umin(32u, h.pagesize / segmentsize);
                g.additional = calc_additional_chunks(h.pagesize, g.fullsegments, segmentsize, chunksize);
                g.segments = g.fullsegments + (g.additional > 0u ? 1u : 0u);
                g.capacity = g.fullsegments * 32u + g.additional;
            }
            else
            {
                g.fullsegments = g.additional = g.segments = 0u;
                g.capacity = umin(h.pagesize / chunksize, 32u);
            }
            return g;
        }

        /* Capacity of a page formatted with chunksize. */
        __device__ __forceinline__ u32 page_capacity(const mmc_device_handle& h, u32 chunksize)
        {
            return chunk_geom(h, chunksize).capacity;
        }

        /* Claim one chunk on a page whose fill slot is reserved:
         * addChunkHierarchy (Scatter.hpp:397-421) for hierarchical pages,
         * addChunkNoHierarchy (:432-443) otherwise. Both begin with one atomicOr
         * on a per-lane word (a segment's on-page mask or the page bitmask), so
         * the lanes of a warp issue that first claim as a single instruction
         * whatever their page kind; a lane that loses the race continues the
         * reference's exact retry sequence. `mask` is the page's segment hints. */
        template<class Ids>
        __device__ void* claim_chunk(const mmc_device_handle& h, u32 page, u32 chunksize, const ChunkGeom& g, u32 mask)
        {
            u32* word;
            u32 spots;
            u32 seg = 0u;
            u32 tries = 1u;
            u32* onpagemasks = nullptr;
            if(g.hier)
            {
                seg = Ids::laneid() % g.segments;
                if((mask & (1u << seg)) != 0u)
                    seg = nextspot(mask, seg, g.segments);
                tries = g.segments - static_cast<u32>(__popc(mask));
                onpagemasks = on_page_masks(h, page, g.segments);
                word = onpagemasks + seg;
                spots = seg < g.fullsegments ? 32u : g.additional;
            }
            else
            {
                word = &h.bitmask[page];
                spots = g.capacity;
            }
            if(tries == 0u)
                return nullptr;
            const u32 spot = Ids::laneid() % spots;
            const u32 bit = 1u << spot;
            const u32 old = atomicOr(word, bit);
            int got = (old & bit) == 0u ? static_cast<int>(spot) : usespot_continue(word, spots, spot, old);
            if(!g.hier)
                return got == -1 ? nullptr : page_data(h, page) + static_cast<u32>(got) * chunksize;
            for(u32 i = 0;;)
            {
                if(got != -1)
                    return page_data(h, page) + (32u * seg + static_cast<u32>(got)) * chunksize;
                atomicOr(&h.bitmask[page], 1u << seg);
                /* A free in this segment may have cleared the hint just before
                 * it was set; undo a mark the segment no longer deserves so no
                 * stale "full" bit outlives the chunks. A lone thread only gets
                 * here for a full segment, so this never fires serially. */
                if(static_cast<u32>(__popc(ld_rlx(&onpagemasks[seg]))) < spots)
                    atomicAnd(&h.bitmask[page], ~(1u << seg));
                seg = nextspot(mask, seg, g.segments);
                if(++i >= tries)
                    return nullptr;
                spots = seg < g.fullsegments ? 32u : g.additional;
                got = usespot<Ids>(&onpagemasks[seg], spots);
            }
        }

        /* tryUsePage, Scatter.hpp:454-518; [lo, hi] is isChunkSizeInRange (:586-588). */
        template<class Ids>
        __device__ void* try_use_page(const mmc_device_handle& h, u32 page, u32 chunksize, u32 lo, u32 hi)
        {
            void* chunk_ptr = nullptr;
            /* the segment hints are read before the fill-count atomic so both
             * round trips overlap (the reference reads them just after it,
             * Scatter.hpp:404; alone on the heap both reads see the same word) */
            u32 mask = chunksize <= h.hierarchyThreshold ? ld_rlx(&h.bitmask[page]) : 0u;
            const u32 filllevel = atomicAdd(&h.count[page], 1u);
            const bool reset = Ids::reset(h) != 0u;
            bool tryAllocMem = !reset;
            if(reset && filllevel < h.pagesize)
            {
                const u32 oldChunksize = atomicCAS(&h.chunksize[page], 0u, chunksize);
                if(oldChunksize == 0u)
                    freemap_clear_acked(h.freemap, page); /* our fill slot keeps the page from a reset */
                if(oldChunksize == 0u || (oldChunksize >= lo && oldChunksize <= hi))
                    tryAllocMem = true;
                if(oldChunksize != 0u && oldChunksize != chunksize)
                {
                    chunksize = oldChunksize;
                    mask = ld_rlx(&h.bitmask[page]);
                }
            }
            if(tryAllocMem)
            {
                const ChunkGeom g = chunk_geom(h, chunksize);
                if(filllevel < g.capacity)
                    chunk_ptr = claim_chunk<Ids>(h, page, chunksize, g, mask);
            }
            if(chunk_ptr == nullptr)
                atomicSub(&h.count[page], 1u);
            return chunk_ptr;
        }

        /* One page of allocChunked's walk (Scatter.hpp:580-604), given the page's
         * chunk size as already loaded. The reference's CAS(0 -> minAllocation)
         * only writes a zero word; on a formatted page it just returns the value,
         * so it is issued only when the load saw zero. */
        template<class Ids>
        __device__ __forceinline__ void* attempt_page(const mmc_device_handle& h, u32 page, u32 before, u32 bytes,
                                                      u32 minAllocation, u32 maxchunksize)
        {
            if(before == 0u)
            {
                freemap_clear_acked(h.freemap, page);
                before = atomicCAS(&h.chunksize[page], 0u, minAllocation);
            }
            u32 use = 0u;
            if(before == 0u)
                use = minAllocation;
            else if(before >= bytes && before <= maxchunksize)
                use = before;
            if(use == 0u)
            {
                MMC_STAT(h, MMC_STAT_SIZE_MISMATCH);
                return nullptr;
            }
            void* r = try_use_page<Ids>(h, page, use, bytes, maxchunksize);
            if(r == nullptr)
                MMC_STAT(h, MMC_STAT_PAGE_FULL);
            return r;
        }

        /* The pages of one region a request may use, as two masks in page order
         * (bit i = page region_offset + i): unformatted pages (chunk size 0) and
         * pages formatted with a chunk size in [bytes, maxchunksize]. Every other
         * page is one the reference's walk visits only to find it formatted for
         * another size or taken by a multi-page run (Scatter.hpp:584-591). The
         * chunk-size words are read with 16-byte loads, 16 pages in flight at
         * once. Needs regionsize % 4 == 0 and regionsize <= 32. */
        __device__ __forceinline__ void region_candidates(const mmc_device_handle& h, u32 region_offset, u32 bytes,
                                                          u32 maxchunksize, u32& zero, u32& fit)
        {
            const u32 R = h.regionsize;
            zero = 0u;
            fit = 0u;
            for(u32 base = 0; base < R; base += 16u)
            {
                uint4 v[4];
#pragma unroll
                for(u32 k = 0; k < 4u; ++k)
                    v[k] = (base + 4u * k < R) ? ld_rlx_v4(&h.chunksize[region_offset + base + 4u * k])
                                               : make_uint4(~0u, ~0u, ~0u, ~0u);
#pragma unroll
                for(u32 k = 0; k < 4u; ++k)
                {
                    const u32 w[4] = {v[k].x, v[k].y, v[k].z, v[k].w};
#pragma unroll
                    for(u32 j = 0; j < 4u; ++j)
                    {
                        const u32 bit = base + 4u * k + j;
                        if(bit < 32u)
                        {
                            zero |= (w[j] == 0u ? 1u : 0u) << bit;
                            fit |= ((w[j] >= bytes && w[j] <= maxchunksize) ? 1u : 0u) << bit;
                        }
                    }
                }
            }
        }

        /* allocChunked's two-pass region walk (Scatter.hpp:563-636), resumed after
         * the first page: in the first region of pass 0 the region counter is
         * the one already read (fill0) and the start page was already tried.
         *
         * That first region is walked page by page, as the reference walks it
         * (most walks end there, after a page or two). Every further region is
         * read whole first (region_candidates: one round trip for 16 pages) and
         * only its usable pages are tried, in the reference's order from the
         * entry page: a walk that crosses regions of full pages or of multi-page
         * runs (the page-based area, where region counters stay low because
         * only failed chunk walks raise them) then costs one round trip per
         * region instead of one per page. The region counters themselves are
         * read eight regions ahead, so a stretch of regions skipped as 3/4 full
         * costs one round trip per eight (a walk only changes the counter of the
         * region it is in). Alone on the heap every page gets the reference's
         * outcome, in the reference's order. */
        template<class Ids>
        __device__ void* alloc_chunked_walk(const mmc_device_handle& h, u32 bytes, u32 minAllocation,
                                            u32 maxchunksize, u32 global_start_page, u32 fill0)
        {
            const u32 R = h.regionsize;
            const u32 numpages = h.numpages;
            const u32 numregions = h.numregions;
            const u32 pagesperblock = h.pagesperblock;
            const bool batched = (R % 4u) == 0u && R <= 32u;
            const u32 rmask = R >= 32u ? 0xFFFFFFFFu : ((1u << R) - 1u);
            constexpr u32 kAhead = 8u;
            u32 checklevel = R * 3u / 4u;
            for(u32 finder = 0; finder < 2u; ++finder)
            {
                u32 global_page = global_start_page;
                u32 ahead[kAhead];
                u32 ahead_left = 0u; /* counters of the next regions already read */
                do
                {
                    const u32 region = global_page / R;
                    const bool resumed = finder == 0u && global_page == global_start_page;
                    if(!resumed && ahead_left == 0u)
                    {
#pragma unroll
                        for(u32 k = 0; k < kAhead; ++k)
                        {
                            u32 r = region + k;
                            r = r >= numregions ? r - numregions : r;
                            ahead[k] = ld_rlx(&h.regions[r]);
                        }
                        ahead_left = kAhead;
                    }
                    u32 regionfilllevel = fill0;
                    if(!resumed)
                    {
                        regionfilllevel = ahead[kAhead - ahead_left];
                        --ahead_left;
                    }
                    const u32 region_offset = region * R;
                    if(regionfilllevel < checklevel)
                    {
                        if(batched && !resumed)
                        {
                            u32 zero, fit;
                            region_candidates(h, region_offset, bytes, maxchunksize, zero, fit);
                            /* rotate so that bit i is the i-th page visited from the entry page */
                            const u32 s0 = global_page - region_offset;
                            const u32 z = s0 == 0u ? zero : (((zero >> s0) | (zero << (R - s0))) & rmask);
                            const u32 f = s0 == 0u ? fit : (((fit >> s0) | (fit << (R - s0))) & rmask);
                            for(u32 todo = z | f; todo != 0u; todo &= todo - 1u)
                            {
                                const u32 i = static_cast<u32>(__ffs(static_cast<int>(todo))) - 1u;
                                const u32 page = region_offset + (s0 + i) % R;
                                MMC_STAT(h, MMC_STAT_WALK_PAGES);
                                const u32 before = ((z >> i) & 1u) ? 0u : ld_rlx(&h.chunksize[page]);
                                void* res = attempt_page<Ids>(h, page, before, bytes, minAllocation, maxchunksize);
                                if(res != nullptr)
                                    return res;
                            }
                        }
                        else
                        {
                            u32 page_in_region = global_page;
                            bool skip = resumed;
                            do
                            {
                                if(!skip)
                                {
                                    MMC_STAT(h, MMC_STAT_WALK_PAGES);
                                    void* res = attempt_page<Ids>(h, page_in_region,
                                                                  ld_rlx(&h.chunksize[page_in_region]), bytes,
                                                                  minAllocation, maxchunksize);
                                    if(res != nullptr)
                                        return res;
                                }
                                skip = false;
                                page_in_region = region_offset + ((page_in_region + 1u) % R);
                            } while(page_in_region != global_page);
                        }

                        if(regionfilllevel + 1u <= R)
                            atomicCAS(&h.regions[region], regionfilllevel, regionfilllevel + 1u);
                        MMC_STAT(h, MMC_STAT_REGION_FAIL);
                    }
                    else
                        MMC_STAT(h, MMC_STAT_REGION_SKIP);
                    global_page = (global_page + R) % numpages;
                    if(global_page % pagesperblock == 0u)
                    {
                        const u32 access_block_id = global_page / pagesperblock;
                        /* racy by design (Scatter.hpp:625-628) */
                        if(access_block_id > ld_rlx(&h.state->firstfreeblock))
                            st_rlx(&h.state->firstfreeblock, access_block_id);
                    }
                } while(global_page != global_start_page);
                checklevel = R + 1u;
            }
            return nullptr;
        }

        /* One page of a same-size group claim, by the group's leader: reserve up
         * to `want` fill slots with one atomicAdd (the reference's per-chunk
         * check, filllevel < capacity, applied to k reservations at once), claim
         * as many free bits of the page's bitmask with atomicOr, give back what
         * found no bit. Pages of chunks above HierarchyThreshold only (their
         * bitmask maps chunks directly). Returns the claimed bits. */
        __device__ __forceinline__ u32 claim_bits_on_page(const mmc_device_handle& h, u32 page, u32 use, u32 want)
        {
            const u32 cap = umin(h.pagesize / use, 32u);
            const u32 old = atomicAdd(&h.count[page], want);
            u32 grant = old < cap ? umin(want, cap - old) : 0u;
            if(grant < want)
                atomicSub(&h.count[page], want - grant);
            const u32 full = cap == 32u ? 0xFFFFFFFFu : ((1u << cap) - 1u);
            u32 mask = grant != 0u ? ld_rlx(&h.bitmask[page]) : full;
            u32 got = 0u;
            for(u32 tries = 0; grant != 0u && tries < MMC_USESPOT_MAX_TRIES; ++tries)
            {
                u32 free = ~mask & full;
                if(free == 0u)
                    break;
                u32 pick = 0u;
                for(u32 n = 0; n < grant && free != 0u; ++n)
                {
                    pick |= free & (0u - free); /* lowest free bit */
                    free &= free - 1u;
                }
                const u32 prev = atomicOr(&h.bitmask[page], pick);
                const u32 mine = pick & ~prev;
                got |= mine;
                grant -= static_cast<u32>(__popc(mine));
                mask = prev | pick;
            }
            if(grant != 0u)
                atomicSub(&h.count[page], grant); /* reserved slots no bit was found for */
            return got;
        }

        /* Same-size claims: lanes of a warp asking for the same size hash to the
         * same first page (the hash depends on the size, the SM and the warp,
         * not the lane), where the reference has each of them reserve a fill
         * slot and claim a bit on its own, all contending for one count word and
         * one bitmask word. Here the lanes are grouped by size (the whole warp
         * when a min/max reduction shows one size, else __match_any_sync, groups
         * of four lanes or more), and the group's lowest lane claims for all of
         * them, page by page through the first region in the walk's order
         * (claim_bits_on_page); the lane of rank r takes the r-th chunk claimed.
         * Lanes left over go the usual way. Measured on GB300: a warp-uniform
         * 256 B / 512 B / 1 KiB stress runs 1.7x / 2.9x / 2.4x faster, the
         * mixed-size stress 2.6 % faster (smaller groups cost more than they
         * save, hence the four-lane floor). Returns true with `out` set when
         * this lane got its chunk. */
        template<class Ids>
        __device__ __forceinline__ bool claim_same_size(const mmc_device_handle& h, u32 bytes, u32 minAllocation,
                                                        u32 maxchunksize, u32 start, u32 fill0, u32 cs0, void*& out)
        {
            if(Ids::reset(h))
                return false;
            const u32 am = __activemask();
            const bool same = __reduce_min_sync(am, bytes) == __reduce_max_sync(am, bytes);
            const u32 peers = same ? am : __match_any_sync(am, bytes);
            const u32 k = static_cast<u32>(__popc(peers));
            /* sizes whose pages could be hierarchical keep the one-lane claim */
            if(k < 4u || minAllocation <= h.hierarchyThreshold)
                return false;
            const u32 lane = Ids::laneid();
            const int leader = __ffs(static_cast<int>(peers)) - 1;
            const bool lead = lane == static_cast<u32>(leader);
            const u32 rank = static_cast<u32>(__popc(peers & lanemask_lt()));
            const u32 R = h.regionsize;
            const u32 region_offset = (start / R) * R;
            const u32 region_ok = __shfl_sync(peers, fill0 < R * 3u / 4u ? 1u : 0u, leader);
            if(region_ok == 0u)
                return false;
            u32 served = 0u;
            u32 page = start;
            for(u32 visited = 0; visited < R && served < k; ++visited)
            {
                u32 got = 0u, use = 0u;
                if(lead)
                {
                    u32 before = visited == 0u ? cs0 : ld_rlx(&h.chunksize[page]);
                    if(before == 0u)
                    {
                        freemap_clear_acked(h.freemap, page);
                        before = atomicCAS(&h.chunksize[page], 0u, minAllocation);
                    }
                    use = before == 0u ? minAllocation : ((before >= bytes && before <= maxchunksize) ? before : 0u);
                    if(use > h.hierarchyThreshold)
                        got = claim_bits_on_page(h, page, use, k - served);
                }
                got = __shfl_sync(peers, got, leader);
                use = __shfl_sync(peers, use, leader);
                const u32 n = static_cast<u32>(__popc(got));
                if(rank >= served && rank < served + n)
                {
                    u32 m = got;
                    for(u32 i = served; i < rank; ++i)
                        m &= m - 1u;
                    const u32 bit = static_cast<u32>(__ffs(static_cast<int>(m))) - 1u;
                    out = page_data(h, page) + bit * use;
                }
                served += n;
                page = region_offset + ((page + 1u) % R);
            }
            if(rank < served)
            {
                MMC_STAT(h, MMC_STAT_FIRST_PAGE);
                return true;
            }
            return false;
        }

        /* allocChunked, Scatter.hpp:527-637. The walk's first page is tried with
         * its region counter and chunk size read together, as straight-line
         * code every lane of a warp executes in step; only lanes whose first
         * page fails enter the (divergent) rest of the walk. */
        template<class Ids>
        __device__ void* alloc_chunked(const mmc_device_handle& h, u32 bytes)
        {
            const u32 P = h.pagesize;
            const u32 R = h.regionsize;
            const u32 minAllocation = umax(bytes, h.paddedMinChunkSize);
            const u32 numpages = h.numpages;
            const u32 pagesperblock = h.pagesperblock;
            const u32 reloff = Ids::warpSize * minAllocation / P;
            const u32 start_page_in_block = (minAllocation * h.hashingK + h.hashingDistMP * Ids::smid()
                                             + (h.hashingDistWP + h.hashingDistWPRel * reloff) * Ids::warpid())
                % pagesperblock;
            const u32 maxchunksize = umin(P, umax(h.wastefactor * bytes, h.paddedMinChunkSize));
            const u32 ffb = Ids::cachedHints ? __ldca(&h.state->firstfreeblock) : ld_rlx(&h.state->firstfreeblock);
            u32 global_start_page = start_page_in_block + ffb * pagesperblock;
            if(global_start_page >= numpages)
                global_start_page %= numpages; /* unreachable for a consistent header; keeps accesses in bounds */

            const u32 fill0 = ld_rlx(&h.regions[global_start_page / R]);
            const u32 cs0 = ld_rlx(&h.chunksize[global_start_page]);
            MMC_STAT(h, MMC_STAT_CHUNKED);
            if constexpr(Ids::warpSize > 1u)
            {
                void* grouped = nullptr;
                if(claim_same_size<Ids>(h, bytes, minAllocation, maxchunksize, global_start_page, fill0, cs0, grouped))
                    return grouped;
            }
            if(fill0 < R * 3u / 4u)
            {
                void* res = attempt_page<Ids>(h, global_start_page, cs0, bytes, minAllocation, maxchunksize);
                if(res != nullptr)
                {
                    MMC_STAT(h, MMC_STAT_FIRST_PAGE);
                    return res;
                }
            }
            void* res = alloc_chunked_walk<Ids>(h, bytes, minAllocation, maxchunksize, global_start_page, fill0);
            if(res == nullptr)
                MMC_STAT(h, MMC_STAT_CHUNKED_FAIL);
            return res;
        }

        /* deallocChunked, Scatter.hpp:646-736 */
        template<class Ids>
        __device__ void dealloc_chunked(const mmc_device_handle& h, void* mem, u32 page, u32 chunksize)
        {
            const u32 P = h.pagesize;
            const u32 inpage_offset = static_cast<u32>(static_cast<char*>(mem) - page_data(h, page));
            u32 segment;
            if(chunksize <= h.hierarchyThreshold)
            {
                const ChunkGeom g = chunk_geom(h, chunksize);
                segment = inpage_offset / (chunksize * 32u);
                const u32 withinsegment = (inpage_offset - segment * (chunksize * 32u)) / chunksize;
                atomicAnd(on_page_masks(h, page, g.segments) + segment, ~(1u << withinsegment));
            }
            else
                segment = inpage_offset / chunksize;
            /* both kinds clear their bit of the page bitmask (:665, :670) */
            atomicAnd(&h.bitmask[page], ~(1u << segment));

            u32 oldfilllevel = 0u;
            if(Ids::reset(h))
            {
                oldfilllevel = atomicCAS(&h.count[page], 1u, P);
                bool locked = oldfilllevel == 1u;
                if(!locked)
                {
                    oldfilllevel = atomicSub(&h.count[page], 1u);
                    /* The reference resets a page only when a freer's CAS sees
                     * count == 1, so two last frees racing past each other leave
                     * it formatted. A freer that took the count from 1 to 0 takes
                     * the same lock (count = pagesize) if nobody has claimed the
                     * page since; a lone thread never gets here with old == 1. */
                    if(oldfilllevel == 1u)
                        locked = atomicCAS(&h.count[page], 0u, P) == 0u;
                }
                if(locked)
                {
                    page_init(h, page);
                    /* no chunk is live under the lock: drop any segment hint a
                     * race left behind (a no-op for the reference's serial runs) */
                    atomicExch(&h.bitmask[page], 0u);
                    if(atomicCAS(&h.chunksize[page], chunksize, 0u) == chunksize)
                        freemap_set(h.freemap, page);
                    __threadfence();
                    atomicSub(&h.count[page], P);
                }
            }
            else
                oldfilllevel = atomicSub(&h.count[page], 1u);

            if(oldfilllevel == P / 2u / chunksize)
            {
                const u32 region = page / h.regionsize;
                atomicExch(&h.regions[region], 0u);
                const u32 block = page / h.pagesperblock;
                if(Ids::warpid() + Ids::laneid() == 0u)
                    atomicMin(&h.state->firstfreeblock, block);
            }
        }

        /* chunk size seen by the page-based scan; index numpages (one past the end,
         * which the reference's second search reads) counts as "in use". */
        __device__ __forceinline__ u32 scan_chunksize(const mmc_device_handle& h, u32 page)
        {
            return page < h.numpages ? ld_rlx(&h.chunksize[page]) : 1u;
        }

        /* markpages, Scatter.hpp:745-764 (the serial form): CAS(chunksize,
         * 0 -> bytes) page by page; on a failure the pages already set are put
         * back with CAS(bytes -> 0). */
        __device__ inline bool markpages(const mmc_device_handle& h, u32 startpage, u32 pages, u32 bytes)
        {
            u32 abord = 0xFFFFFFFFu;
            for(u32 trypage = startpage; trypage < startpage + pages; ++trypage)
            {
                const u32 old = atomicCAS(&h.chunksize[trypage], 0u, bytes);
                if(old != 0u)
                {
                    abord = trypage;
                    break;
                }
            }
            if(abord == 0xFFFFFFFFu)
            {
                freemap_range(h.freemap, startpage, pages, false);
                asm volatile("fence.acq_rel.gpu;" ::: "memory");
                return true;
            }
            for(u32 trypage = startpage; trypage < abord; ++trypage)
                if(atomicCAS(&h.chunksize[trypage], bytes, 0u) == bytes)
                    freemap_set(h.freemap, trypage);
            return false;
        }

        /* allocPageBasedSingleRegion, Scatter.hpp:775-813 */
        __device__ inline void* alloc_page_based_single_region(const mmc_device_handle& h, u32 startpage, u32 endpage,
                                                        u32 bytes)
        {
            const u32 pagestoalloc = divup(bytes, h.pagesize);
            u32 freecount = 0;
            bool left_free = false;
            for(u32 search_page = startpage + 1u; search_page > endpage;)
            {
                --search_page;
                if(scan_chunksize(h, search_page) == 0u)
                {
                    if(++freecount == pagestoalloc)
                    {
                        if(search_page + pagestoalloc <= h.numpages && markpages(h, search_page, pagestoalloc, bytes))
                        {
                            if(!left_free)
                            {
                                /* the reference stores search_page - 1, which wraps for a
                                 * run ending at page 0 (Scatter.hpp:800-804) */
                                u32 nf = search_page - 1u;
                                if(!h.reference_quirks && search_page == 0u)
                                    nf = 0u;
                                atomicCAS(&h.state->firstFreePageBased, startpage, nf);
                            }
                            return page_data(h, search_page);
                        }
                    }
                }
                else
                {
                    left_free = true;
                    freecount = 0;
                }
            }
            return nullptr;
        }

        /* allocPageBasedSingle, Scatter.hpp:824-840, with a bounded, backed-off
         * mutex wait: the reference's serial protocol, used for SerialIds. */
        __device__ inline void* alloc_page_based_single(const mmc_device_handle& h, u32 bytes)
        {
            u32 ns = 32u;
            for(u32 it = 0; atomicExch(&h.state->pagebasedMutex, 1u) != 0u; ++it)
            {
                if(it >= MMC_MUTEX_MAX_SPINS)
                {
                    set_error(h, MMC_DEVERR_TIMEOUT);
                    return nullptr;
                }
                __nanosleep(ns);
                if(ns < 2048u)
                    ns <<= 1;
            }
            __threadfence();
            const u32 spage = ld_rlx(&h.state->firstFreePageBased);
            void* res = alloc_page_based_single_region(h, spage, 0u, bytes);
            if(res == nullptr)
                res = alloc_page_based_single_region(h, h.numpages, spage, bytes);
            __threadfence();
            atomicExch(&h.state->pagebasedMutex, 0u);
            return res;
        }

        /* What the concurrent page-based search needs of the handle. */
        struct PageScan
        {
            u32* chunksize;
            u32* freemap;
            mmc_heap_state* state;
            char* pages;
            u32 numpages;
            u32 pagesize;
            u32 reference_quirks;
        };

        /* markpages (Scatter.hpp:745-764) for concurrent callers. The run's
         * top page is claimed first, alone: searches that meet one free
         * stretch all settle on runs ending at its top page, and that CAS lets
         * exactly one of them go on, while the others lose it holding no page
         * (a claim that lost part way would put back pages that concurrent
         * searches saw taken and settled below, leaving a hole of a page or
         * two that no multi-page run fits). The other pages' CASes go out 4 at
         * a time (independent atomics in flight together, not one round trip
         * per page); on a failure every page this call set is put back with
         * CAS(bytes -> 0), as the reference's roll-back does, and gets its
         * free-page bit back. A run that is marked has its bits cleared (and
         * the clears performed) before it is handed out. With no concurrent
         * caller the outcome is the serial form's, which claims upward. */
        __device__ __forceinline__ bool markpages_batched(const PageScan& c, u32 startpage, u32 pages, u32 bytes,
                                                          u32& free_below, u32& top_owner)
        {
            const u32 end = startpage + pages;
            top_owner = atomicCAS(&c.chunksize[end - 1u], 0u, bytes);
            if(top_owner != 0u)
            {
                /* the pages below the top were free in the search */
                free_below = pages - 1u;
                return false;
            }
            const u32 last = end - 1u;
            for(u32 base = startpage; base < last; base += 4u)
            {
                u32 old[4];
#pragma unroll
                for(u32 k = 0; k < 4u; ++k)
                    old[k] = (base + k < last) ? atomicCAS(&c.chunksize[base + k], 0u, bytes) : 0u;
                u32 lost = 0u;
#pragma unroll
                for(u32 k = 0; k < 4u; ++k)
                    lost |= (old[k] != 0u ? 1u : 0u) << k;
                if(lost != 0u)
                {
                    u32 top_back = 0u; /* highest page put back, plus one */
                    if(atomicCAS(&c.chunksize[last], bytes, 0u) == bytes)
                    {
                        freemap_set(c.freemap, last);
                        top_back = end;
                    }
                    for(u32 trypage = startpage; trypage < base; ++trypage)
                        if(atomicCAS(&c.chunksize[trypage], bytes, 0u) == bytes)
                        {
                            freemap_set(c.freemap, trypage);
                            top_back = umax(top_back, trypage + 1u);
                        }
#pragma unroll
                    for(u32 k = 0; k < 4u; ++k)
                        if(base + k < last && ((lost >> k) & 1u) == 0u
                           && atomicCAS(&c.chunksize[base + k], bytes, 0u) == bytes)
                        {
                            freemap_set(c.freemap, base + k);
                            top_back = umax(top_back, base + k + 1u);
                        }
                    /* Pages put back are freed pages, and a free raises the
                     * search hint over them (deallocPageBased's atomicMax,
                     * Scatter.hpp:885): while this claim held them, concurrent
                     * searches saw them used and may have settled below them
                     * and lowered the hint, which would leave them a hole no
                     * later search visits. */
                    if(top_back != 0u)
                        atomicMax(&c.state->firstFreePageBased, top_back - 1u);
                    /* the pages from startpage up to the lowest lost one were free */
                    free_below = base + static_cast<u32>(__ffs(static_cast<int>(lost))) - 1u - startpage;
                    return false;
                }
            }
            freemap_range(c.freemap, startpage, pages, false);
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            return true;
        }

        constexpr u32 kNoRun = 0xFFFFFFFFu;
        /* lost runs a concurrent multi-page search looks at again before it
         * settles below them */
        constexpr u32 kLostRunRetries = 8u;

        /* Bits b_hi down to b_lo of free-page word w (value x), continuing a
         * downward count of consecutive free pages: returns the first page of
         * a run of n free pages once the count reaches n, else kNoRun. A used
         * page resets the count; one that ends a stretch of two or more free
         * pages the search could not use marks those pages as left behind
         * (left_free), which keeps the search from lowering the hint past
         * them. A single free page between used ones is not counted: no
         * multi-page run (two pages at least) can use it until a neighbour is
         * freed, and that free raises the hint again. (The
         * reference marks every used page, so its hint also stays above
         * stretches of used pages it passed. Lowering it past those spares
         * every later search the rescan and moves no placement while the pages
         * stay used; a run freed there raises the hint again. Only a chunk
         * page reset to free there under resetfreedpages, which raises no
         * hint, is then found by the search from the top instead.) */
        __device__ __forceinline__ u32 scan_freemap_word(u32 x, u32 w, u32 b_hi, u32 b_lo, u32 n, u32& freecount,
                                                         bool& left_free)
        {
            const u32 span = b_hi - b_lo + 1u;
            const u32 mask = span == 32u ? 0xFFFFFFFFu : ((1u << span) - 1u) << b_lo;
            const u32 xm = x & mask;
            if(xm == mask)
            {
                if(freecount + span >= n)
                    return 32u * w + b_hi - (n - freecount - 1u);
                freecount += span;
                return kNoRun;
            }
            if(xm == 0u)
            {
                left_free = left_free || freecount > 1u;
                freecount = 0u;
                return kNoRun;
            }
            for(u32 b = b_hi + 1u; b-- > b_lo;)
            {
                if((xm >> b) & 1u)
                {
                    if(++freecount == n)
                        return 32u * w + b;
                }
                else
                {
                    left_free = left_free || freecount > 1u;
                    freecount = 0u;
                }
            }
            return kNoRun;
        }

        /* allocPageBasedSingleRegion's search (Scatter.hpp:775-813) for concurrent
         * callers, without the global mutex. It visits the pages the reference
         * visits, startpage down to endpage, and counts free runs as the
         * reference counts them (downward, reset at a used page), but reads the
         * free-page bitmap: 16 words, 512 pages, per round trip, with whole
         * words of free or used pages taken in one step. markpages' CAS on the
         * chunk sizes decides who owns a run, top page first. A lane that
         * loses the top page learns the winner's size from the CAS and goes on
         * right below the winner's run (every search that met the same free
         * stretch settled on a run ending at its top page), from the bitmap
         * words it has already read: the lanes that meet one stretch together
         * pack their runs into it one below the other, with no page left
         * between them, as the reference's serial search would. A lane that
         * loses a page below the top (a claim that settled elsewhere) looks
         * at the run again a few times, since that claim may be put back,
         * then keeps counting below the lost page. The hint is lowered as the
         * reference lowers it, to just below the run by a CAS from the value
         * the search started at, when the search left no free page behind.
         * With no concurrent caller this finds the reference's run. */
        __device__ __forceinline__ char* alloc_page_based_scan(const PageScan& c, u32 startpage, u32 endpage,
                                                               u32 bytes)
        {
            const u32 n = divup(bytes, c.pagesize);
            u32 freecount = 0u;
            bool left_free = false;
            u32 retries = 0u;
            const u32 wend = endpage >> 5;
            /* pages top-1, top-2, ..., endpage remain (top wraps to 0 for the
             * reference's underflowed hint: then nothing is visited); a start
             * past page numpages, which no consistent hint holds, is cut to it
             * so every bitmap word read lies inside the map */
            if(startpage > c.numpages && startpage != 0xFFFFFFFFu)
                startpage = c.numpages;
            u32 top = startpage + 1u;
            u32 g0 = 0u;
            uint4 grp[4];
            bool reuse = false; /* the window read last still holds word whi */
            while(top > endpage)
            {
                const u32 whi = (top - 1u) >> 5;
                if(!(reuse && whi <= g0 + 3u && whi + 12u >= g0))
                {
                    g0 = whi & ~3u; /* 16-byte group holding word whi */
#pragma unroll
                    for(u32 k = 0; k < 4u; ++k)
                        grp[k] = (g0 >= 4u * k && g0 - 4u * k + 3u >= wend)
                                     ? __ldcg(reinterpret_cast<const uint4*>(c.freemap + (g0 - 4u * k)))
                                     : make_uint4(0u, 0u, 0u, 0u);
                }
                reuse = false;
                u32 q = kNoRun;
                u32 wl = whi; /* lowest word scanned */
                /* Not unrolled: ptxas fits the registers of every kernel that
                 * calls malloc around this out-of-line search's own, and the
                 * unrolled loop (the window held in registers) made the
                 * uniform stress kernel spill and run 17 % slower. */
#pragma unroll 1
                for(u32 j = 0; j < 16u; ++j)
                {
                    if(g0 + 3u < j)
                        break; /* below word 0 */
                    const u32 w = g0 + 3u - j;
                    if(w > whi)
                        continue;
                    if(w < wend)
                        break;
                    const uint4 G = grp[j / 4u];
                    const u32 comp = 3u - (j % 4u);
                    const u32 x = comp == 3u ? G.w : (comp == 2u ? G.z : (comp == 1u ? G.y : G.x));
                    wl = w;
                    if(x == 0u)
                        MMC_STAT(c, MMC_STAT_PAGE_SCAN_USED);
                    q = scan_freemap_word(x, w, w == whi ? ((top - 1u) & 31u) : 31u, w == wend ? (endpage & 31u) : 0u,
                                          n, freecount, left_free);
                    if(q != kNoRun)
                        break;
                }
                MMC_STAT_ADD(c, MMC_STAT_PAGE_SCAN, 32u * (whi - wl + 1u));
                if(q == kNoRun)
                {
                    top = wl == wend ? endpage : 32u * wl;
                    continue;
                }
                u32 free_below = 0u, top_owner = 0u;
                if(q + n <= c.numpages && markpages_batched(c, q, n, bytes, free_below, top_owner))
                {
                    if(!left_free)
                    {
                        /* the reference stores q - 1, which wraps for a run
                         * ending at page 0 (Scatter.hpp:800-804) and leaves
                         * every later search empty; fixed mode stores 0 */
                        const u32 nf = (!c.reference_quirks && q == 0u) ? 0u : q - 1u;
                        atomicCAS(&c.state->firstFreePageBased, startpage, nf);
                    }
                    return c.pages + static_cast<u64>(q) * c.pagesize;
                }
                MMC_STAT(c, MMC_STAT_PAGE_LOST);
                if(top_owner != 0u)
                {
                    /* The run's top page went to a concurrent claim: a chunk
                     * page, or a run of top_owner bytes, which in the common
                     * case ends at that page (the searches that meet one free
                     * stretch settle on runs ending at its top). Go on below
                     * it, without waiting for its claim to show in the map. */
                    const u32 skip = top_owner > c.pagesize ? divup(top_owner, c.pagesize) : 1u;
                    const u32 qt = q + n; /* lost top page, plus one */
                    top = qt > skip ? qt - skip : 0u;
                    freecount = 0u;
                    reuse = true;
                    continue;
                }
                if(retries < kLostRunRetries)
                {
                    /* Look at the run's pages again, after a short backoff:
                     * the claim that beat this one may itself lose elsewhere
                     * and put its pages back, and two searches that take each
                     * other's pages both lose. Going on below the lost page at
                     * once would leave the top of the contested stretch to a
                     * later search that may never come (a hole of a page or
                     * two among the runs); the page above the run is used (or
                     * above the start), so counting restarts from 0 there. */
                    __nanosleep(64u << umin(retries, 4u));
                    ++retries;
                    top = q + n;
                    freecount = 0u;
                    continue;
                }
                /* the run below the lost page is still free: keep counting it,
                 * from the page below q */
                freecount = free_below;
                left_free = true;
                top = q;
            }
            return nullptr;
        }

        /* allocPageBased, Scatter.hpp:848-866, for concurrent callers: every
         * lane searches at once, lock-free (alloc_page_based_scan), where the
         * reference's mutex serialises every large request of the GPU and each
         * search walks the page table one round trip per page. Out of line (with
         * its context by value): kept out of every kernel body that calls malloc,
         * the multi-page code no longer crowds the instruction cache of the
         * chunk path; that measured 12 % faster on the uniform stress. */
        __device__ __noinline__ inline char* alloc_page_based_concurrent(const PageScan c, u32 bytes)
        {
            const u32 spage = ld_rlx(&c.state->firstFreePageBased);
            char* res = alloc_page_based_scan(c, spage, 0u, bytes);
            if(res == nullptr)
                res = alloc_page_based_scan(c, c.numpages, spage, bytes);
            if(res == nullptr)
                MMC_STAT(c, MMC_STAT_PAGE_BASED_FAIL);
            return res;
        }

        /* allocPageBased, Scatter.hpp:848-866. Alone on the heap (SerialIds) this
         * is the reference's mutex-serialised search. */
        template<class Ids>
        __device__ void* alloc_page_based(const mmc_device_handle& h, u32 bytes)
        {
            if(Ids::warpSize == 1u)
                return alloc_page_based_single(h, bytes);
            return alloc_page_based_concurrent(
                PageScan{h.chunksize, h.freemap, h.state, h.pages, h.numpages, h.pagesize, h.reference_quirks}, bytes);
        }

        /* deallocPageBased, Scatter.hpp:874-886 (out of line, as the search) */
        __device__ __noinline__ inline void dealloc_page_based(const mmc_device_handle h, u32 page, u32 bytes)
        {
            const u32 pages = divup(bytes, h.pagesize);
            const u32 end = umin(page + pages, h.numpages);
            for(u32 p = page; p < end; ++p)
                page_init(h, p);
            __threadfence();
            for(u32 p = page; p < end; ++p)
                atomicCAS(&h.chunksize[p], bytes, 0u);
            freemap_range(h.freemap, page, end - page, true);
            atomicMax(&h.state->firstFreePageBased, page + pages - 1u);
        }

        /* create, Scatter.hpp:895-912 */
        template<class Ids>
        __device__ __forceinline__ void* create(const mmc_device_handle& h, u32 bytes)
        {
            if(bytes == 0u)
                return nullptr;
            if(bytes <= h.pagesize)
                return alloc_chunked<Ids>(h, bytes);
            if constexpr(!Ids::pageBased)
            {
                set_error(h, MMC_DEVERR_PAGEBASED);
                return nullptr;
            }
            else
            {
                MMC_STAT(h, MMC_STAT_PAGE_BASED);
                return alloc_page_based<Ids>(h, bytes);
            }
        }

        /* 64-bit division for page sizes that are not powers of two, kept out of line */
        __device__ __noinline__ inline u32 page_of_offset_slow(u64 offset, u32 pagesize)
        {
            return static_cast<u32>(offset / pagesize);
        }

        /* destroy, Scatter.hpp:918-946. A pointer outside the pool or on a page
         * without a chunk size (where the reference would divide by zero) is
         * recorded as MMC_DEVERR_BADFREE and ignored.
         *
         * Release: every access this thread made to the block is performed
         * before the atomics that hand the block to a next owner, by a release
         * fence ahead of them; the fence is cumulative, so it also covers what
         * other lanes of the warp did to the block before a __syncwarp this
         * thread passed (a warp-cooperative pattern's writes and reads). Every
         * lane fences before the lanes that free parts of one chunk meet at a
         * __syncwarp, so each lane's accesses to its part are performed before
         * the one grouped decrement. The reference's free has no such fence;
         * without it a thread's last reads of the block can be served after a
         * next owner's writes (a per-thread write/verify/free stress on GB300
         * read foreign data in 1 to 6 of 25 runs, none with the fence). */
        template<class Ids>
        __device__ void destroy(const mmc_device_handle& h, void* mem)
        {
            if(mem == nullptr)
                return;
            const u32 P = h.pagesize;
            const u64 offset = static_cast<u64>(static_cast<char*>(mem) - h.pages);
            if(offset >= static_cast<u64>(h.numpages) * P)
            {
                set_error(h, MMC_DEVERR_BADFREE);
                return;
            }
            const u32 page = (P & (P - 1u)) == 0u ? static_cast<u32>(offset >> (__ffs(static_cast<int>(P)) - 1))
                                                  : page_of_offset_slow(offset, P);
            /* The page's chunk size cannot change while this thread holds a
             * block on it: it is loaded first, and its round trip overlaps the
             * release fence's wait below instead of following it. */
            const u32 chunksize = ld_rlx(&h.chunksize[page]);
            release_fence();
            if(chunksize == 0u)
            {
                set_error(h, MMC_DEVERR_BADFREE);
                return;
            }
            const u32 inpage_offset = static_cast<u32>(offset - static_cast<u64>(page) * P);
            const u32 block = inpage_offset / chunksize;
            const u32 inblockoffset = inpage_offset - block * chunksize;
            if(inblockoffset != 0u)
            {
                /* XMallocSIMD sub-allocation: the lane count lives at the chunk head.
                 * Lanes freeing parts of the same chunk together subtract as one
                 * (the lowest of them, after a __syncwarp that every lane
                 * reaches after its own release fence); whoever takes the count
                 * to zero frees the chunk, as each lane's own decrement would. */
                u32* counter = reinterpret_cast<u32*>(page_data(h, page) + block * chunksize);
                u32 sub = 1u;
                if constexpr(Ids::warpSize > 1u)
                {
                    const u32 peers
                        = __match_any_sync(__activemask(), reinterpret_cast<unsigned long long>(counter));
                    __syncwarp(peers);
                    if(Ids::laneid() != static_cast<u32>(__ffs(static_cast<int>(peers))) - 1u)
                        return;
                    sub = static_cast<u32>(__popc(peers));
                }
                const u32 old = atomicSub(counter, sub);
                if(old != sub)
                    return;
                mem = counter;
            }
            if(chunksize < P || (!h.reference_quirks && chunksize == P))
                dealloc_chunked<Ids>(h, mem, page, chunksize);
            else
                dealloc_page_based(h, page, chunksize);
        }

        /* OOM policy: ReturnNull::handleOOM (ReturnNull.hpp:48-51); MMC_OOM_FLAG
         * records the failure instead of BadAllocException's device assert. */
        template<class Ids>
        __device__ __forceinline__ void* handle_oom(const mmc_device_handle& h, void* mem, u32 req)
        {
            if(req != 0u && mem == nullptr && Ids::oom(h) == MMC_OOM_FLAG)
                set_error(h, MMC_DEVERR_OOM);
            return (req != 0u && mem == nullptr) ? nullptr : mem;
        }

        /* DeviceAllocator::malloc (device_allocator.hpp:72-82) with XMallocSIMD's
         * collect/distribute (XMallocSIMD.hpp:118-176): every active lane whose
         * padded size is in (0, pagesize/32) joins one allocation of
         * 16 + sum(sizes); the lowest such lane requests it, writes the lane
         * count at its head (the refcount destroy() decrements, Scatter.hpp:931-940)
         * and each lane receives base + 16 + (sizes of lower lanes). */
        template<class Ids>
        __device__ void* malloc(const mmc_device_handle& h, size_t bytes_in)
        {
            const u32 bytes = apply_padding(Ids::alignment(h), static_cast<u32>(bytes_in));
            if(!Ids::coalesce || Ids::distribution(h) != MMC_DIST_XMALLOCSIMD)
            {
                void* p = create<Ids>(h, bytes);
                return handle_oom<Ids>(h, p, bytes);
            }
            const u32 active = __activemask();
            const bool coalescible = bytes > 0u && bytes < (h.pagesize / 32u);
            const u32 cmask = __ballot_sync(active, coalescible);
            const u32 threadcount = static_cast<u32>(__popc(cmask));
            if(threadcount <= 1u)
            {
                void* p = create<Ids>(h, bytes);
                return handle_oom<Ids>(h, p, bytes);
            }
            /* exclusive prefix of the coalescible lanes' sizes, in lane order */
            const u32 lane = Ids::laneid();
            const u32 mine = coalescible ? bytes : 0u;
            u32 before = 0u;
            if(active == 0xFFFFFFFFu)
            {
                u32 incl = mine;
#pragma unroll
                for(u32 off = 1u; off < 32u; off <<= 1)
                {
                    const u32 v = __shfl_up_sync(0xFFFFFFFFu, incl, off);
                    if(lane >= off)
                        incl += v;
                }
                before = incl - mine;
            }
            else
            {
                for(u32 m = cmask; m != 0u; m &= m - 1u)
                {
                    const u32 src = static_cast<u32>(__ffs(static_cast<int>(m))) - 1u;
                    const u32 v = __shfl_sync(active, mine, static_cast<int>(src));
                    if(src < lane)
                        before += v;
                }
            }
            const u32 total = __reduce_add_sync(active, mine);
            const u32 leader = static_cast<u32>(__ffs(static_cast<int>(cmask))) - 1u;
            u32 req = bytes;
            if(coalescible)
                req = (lane == leader) ? 16u + total : 0u;
            void* mem = create<Ids>(h, req);
            mem = handle_oom<Ids>(h, mem, req);
            if(coalescible && lane == leader && mem != nullptr)
            {
                st_rlx(static_cast<u32*>(mem), threadcount);
                /* The count's sector is usually cold, and the store leaves it
                 * partly valid in L2: the frees' atomics on it would wait for
                 * the DRAM fill. Fetch it now, while the lanes use their parts. */
                asm volatile("prefetch.global.L2 [%0];" ::"l"(mem));
            }
            /* The lane count must be seen by every later free of a sub-allocation
             * (device-scope atomicSubs on this word). The warp barrier orders
             * the leader's store before every lane's accesses after it, the
             * frees included; a free by another thread is ordered through the
             * synchronisation that handed it the pointer. (The reference stores
             * the count with a block-scope fence, XMallocSIMD.hpp:160-166; a
             * device-scope fence here measured 3-5 % slower on the batched
             * workload.) */
            __syncwarp(active);
            const unsigned long long base
                = __shfl_sync(active, reinterpret_cast<unsigned long long>(mem), static_cast<int>(leader));
            if(!coalescible)
                return mem;
            return base != 0ull ? reinterpret_cast<char*>(base) + 16u + before : nullptr;
        }

        template<class Ids>
        __device__ __forceinline__ void free(const mmc_device_handle& h, void* p)
        {
            destroy<Ids>(h, p);
        }

        /* For a caller about to free a block whose contents are dead: drop the
         * whole 128-byte lines inside [p, p + bytes) from L2 without writing
         * them back to DRAM (discard.global.L2; their bytes become
         * indeterminate), and return p, to be freed. Partial lines at the
         * ends are left alone (they may hold a neighbouring block). No
         * counterpart in the reference: a short-lived block's payload
         * otherwise costs a DRAM write-back after it is freed.
         *
         * Why no later owner's data can be discarded. In the PTX memory model
         * a discard is a weak write of indeterminate bytes to each line. The
         * free that follows issues a fence.release.gpu in every lane ahead of
         * the relaxed device-scope atomics that release the chunk, which
         * orders the discards (and every earlier access of the thread to the
         * block, including what other lanes of the warp wrote into it before a
         * __syncwarp this thread passed) before those atomics: a fence followed
         * by a strong write is a release pattern. A later owner can reach the block only
         * through an atomic that reads what those atomics wrote, and its
         * accesses to the block take their address from that atomic's result,
         * so they reach L2 after the discards. (A dependent read of each
         * discarded line, the other way to order them, misses L2 and measured
         * 17 % slower on the stress.) Call it right before the free. */
        __device__ __forceinline__ void* discard_dead_block(void* p, u32 bytes)
        {
            const u64 a = reinterpret_cast<u64>(p);
            const u64 lo = (a + 127ull) & ~127ull;
            const u64 end = a + bytes;
            for(u64 x = lo; x + 128ull <= end; x += 128ull)
                asm volatile("discard.global.L2 [%0], 128;" ::"l"(x) : "memory");
            return p;
        }

        /* ------------------------------------------------ free-slot counting */

        /* Run summary of a page range for the multi-page slot count: the
         * reference's serial scan (Scatter.hpp:1196-1217) counts
         * floor(L / pagestoalloc) per maximal run of L free pages; runs are
         * combined associatively so ranges can be scanned in parallel. */
        struct RunSum
        {
            u32 len; /* pages covered */
            u32 pre; /* free pages at the low end (== len if all free) */
            u32 suf; /* free pages at the high end */
            u32 cnt; /* slots in runs touching neither end */
        };

        __host__ __device__ __forceinline__ RunSum run_leaf(bool free_page)
        {
            return RunSum{1u, free_page ? 1u : 0u, free_page ? 1u : 0u, 0u};
        }
        __host__ __device__ __forceinline__ RunSum run_empty() { return RunSum{0u, 0u, 0u, 0u}; }

        /* a covers lower page indices than b */
        __host__ __device__ __forceinline__ RunSum run_combine(RunSum a, RunSum b, u32 n)
        {
            if(a.len == 0u)
                return b;
            if(b.len == 0u)
                return a;
            const bool af = a.pre == a.len;
            const bool bf = b.pre == b.len;
            RunSum r;
            r.len = a.len + b.len;
            if(af && bf)
            {
                r.pre = r.suf = r.len;
                r.cnt = 0u;
            }
            else if(af)
            {
                r.pre = a.len + b.pre;
                r.suf = b.suf;
                r.cnt = b.cnt;
            }
            else if(bf)
            {
                r.pre = a.pre;
                r.suf = a.suf + b.len;
                r.cnt = a.cnt;
            }
            else
            {
                r.pre = a.pre;
                r.suf = b.suf;
                r.cnt = a.cnt + b.cnt + (a.suf + b.pre) / n;
            }
            return r;
        }

        __host__ __device__ __forceinline__ u32 run_total(RunSum s, u32 n)
        {
            if(s.len != 0u && s.pre == s.len)
                return s.len / n;
            return s.cnt + s.pre / n + s.suf / n;
        }

        __device__ __forceinline__ RunSum shfl_runsum(u32 mask, RunSum s, int src)
        {
            RunSum r;
            r.len = __shfl_sync(mask, s.len, src);
            r.pre = __shfl_sync(mask, s.pre, src);
            r.suf = __shfl_sync(mask, s.suf, src);
            r.cnt = __shfl_sync(mask, s.cnt, src);
            return r;
        }

        /* Free slots of size slot on one page: getAvailaibleSlotsDeviceFunction's
         * single-page branch (Scatter.hpp:1164-1193) with countFreeChunksInPage
         * (:1112-1139). capZero = capacity at max(slot, paddedMinChunkSize). */
        __device__ __forceinline__ u32 page_free_slots(const mmc_device_handle& h, u32 chunksize, u32 count,
                                                       u32 slot, u32 maxchunksize, u32 slotChunk, u32 capSlotChunk)
        {
            if(chunksize >= slot && chunksize <= maxchunksize)
                return (chunksize == slotChunk ? capSlotChunk : page_capacity(h, chunksize)) - count;
            if(chunksize == 0u)
                return capSlotChunk - count;
            return 0u;
        }

        /* handle.getAvailableSlots (device_allocator.hpp:98-106 ->
         * getAvailableSlotsAccelerator, Scatter.hpp:1311-1352): the lanes active
         * at the call share the scan and all of them receive the count. Unlike
         * the reference it needs no block-wide barrier, so any subset of threads
         * may call it. slotSize is padded first (device_allocator.hpp:103). */
        template<class Ids>
        __device__ unsigned available_slots(const mmc_device_handle& h, size_t slotSize_in)
        {
            const u32 slot = apply_padding(Ids::alignment(h), static_cast<u32>(slotSize_in));
            if(slot == 0u)
                return 0u;
            u32 active = 1u, rank = 0u, nact = 1u;
            if(Ids::warpSize > 1u)
            {
                active = __activemask();
                nact = static_cast<u32>(__popc(active));
                rank = static_cast<u32>(__popc(active & lanemask_lt()));
            }
            const u32 P = h.pagesize;
            u32 partial = 0u;
            if(slot < P)
            {
                const u32 maxchunksize = umin(P, h.wastefactor * slot);
                const u32 slotChunk = umax(slot, h.paddedMinChunkSize);
                const u32 capSlotChunk = page_capacity(h, slotChunk);
                for(u32 pg = rank; pg < h.numpages; pg += nact)
                    partial += page_free_slots(h, ld_rlx(&h.chunksize[pg]), ld_rlx(&h.count[pg]), slot, maxchunksize,
                                               slotChunk, capSlotChunk);
                if(Ids::warpSize > 1u)
                    partial = __reduce_add_sync(active, partial);
                return partial;
            }
            /* multi-page slots: each active lane summarises a contiguous range,
             * the summaries are combined in lane order */
            const u32 n = divup(slot, P);
            const u32 per = divup(h.numpages, nact);
            const u32 b = umin(rank * per, h.numpages);
            const u32 e = umin(b + per, h.numpages);
            RunSum s = run_empty();
            for(u32 pg = b; pg < e; ++pg)
                s = run_combine(s, run_leaf(ld_rlx(&h.chunksize[pg]) == 0u), n);
            if(Ids::warpSize > 1u)
            {
                /* ordered fold over the active lanes, result broadcast */
                RunSum acc = run_empty();
                for(u32 m = active; m != 0u; m &= m - 1u)
                {
                    const int src = __ffs(static_cast<int>(m)) - 1;
                    acc = run_combine(acc, shfl_runsum(active, s, src), n);
                }
                s = acc;
            }
            return run_total(s, n);
        }
    } // namespace dev
} // namespace mmc

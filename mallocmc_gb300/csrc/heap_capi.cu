/* heap_capi.cu — heap lifetime, layout, initialisation, free-slot counting and
 * introspection behind the C ABI in include/mallocmc_gb300.h.
 *
 * HBM layout of a heap (identical page offsets and numpages to the reference,
 * Scatter.hpp:962-1019):
 *   pool + 0                      page 0 .. page numpages-1 (pagesize bytes each;
 *                                 the last maxOnPageMasks words of a page hold its
 *                                 on-page masks while it serves chunks <= HierarchyThreshold)
 *   pool + numpages*pagesize      u32 chunksize[numpages]   (page-table word 0)
 *                                 u32 count[numpages]       (word 1)
 *                                 u32 bitmask[numpages]     (word 2)
 *   then                          u32 regions[numregions]
 * The reference stores the same 12 bytes per page as an array of structs; the
 * three-array form keeps every scan and every CAS walk on consecutive words.
 * A separate 512-byte device block holds the mutable header words
 * (mmc_heap_state) and the free-slot scan's partial sums follow it.
 */
#include "mmc_internal.h"

#include <cuda.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <sstream>
#include <string>

namespace
{
    thread_local std::string g_last_error;

    constexpr unsigned kScanThreads = 256;
    constexpr unsigned kMaxScanBlocks = 152u * 8u;

    struct SlotPartial
    {
        uint32_t len, pre, suf, cnt; /* RunSum, or {0, 0, 0, sum} for the single-page branch */
    };
} // namespace

struct mmc_heap
{
    mmc_config cfg;
    int device;
    void* pool_raw;   /* what was allocated / given */
    size_t pool_raw_bytes;
    bool owns_pool;
    char* pool;       /* after Shrink::alignPool */
    size_t memsize;
    char* devblock;   /* mmc_heap_state + slot partials + result word */
    uint32_t* freemap; /* free-page bitmap (mmc_device_handle::freemap) */
    size_t freemap_words; /* words allocated */
    mmc_heap_state* state;
    SlotPartial* partials;
    unsigned* result_word;
    unsigned* host_result; /* pinned */
    mmc_geometry geom;
    mmc_device_handle handle;
    unsigned scan_blocks;
};

namespace mmc
{
    namespace host
    {
        mmc_status fail(mmc_status st, const std::string& msg)
        {
            g_last_error = msg;
            return st;
        }

        mmc_status cuda_check(cudaError_t e, const char* what)
        {
            if(e == cudaSuccess)
                return MMC_OK;
            return fail(MMC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
        }

        unsigned scan_grid(int device)
        {
            int sms = 0;
            if(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0)
                sms = 152;
            return std::min<unsigned>(static_cast<unsigned>(sms) * 4u, kMaxScanBlocks);
        }

        unsigned* slots_result_word(mmc_heap* heap) { return heap->result_word; }
    } // namespace host
} // namespace mmc

using namespace mmc::host;
using mmc::dev::RunSum;

/* ------------------------------------------------------------------ kernels */

/* initDeviceFunction's zeroing (Scatter.hpp:1026-1032) for the page tails, and
 * the header words (:1034-1044). The page-table and region arrays are zeroed
 * with cudaMemsetAsync before this kernel. */
__global__ void mmc_init_kernel(mmc_device_handle h, uint32_t freemap_words)
{
    /* every page starts free: its bit set; bits past numpages stay clear, so
     * the multi-page search sees them (and page numpages) as used */
    for(uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < freemap_words; w += gridDim.x * blockDim.x)
    {
        const uint32_t first = w * 32u;
        h.freemap[w] = first >= h.numpages ? 0u
                                           : (h.numpages - first >= 32u ? 0xFFFFFFFFu
                                                                         : (1u << (h.numpages - first)) - 1u);
    }
    const uint32_t n = h.maxOnPageMasks;
    const uint64_t total = static_cast<uint64_t>(h.numpages) * n;
    for(uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < total;
        i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        const uint32_t page = static_cast<uint32_t>(i / n);
        const uint32_t w = static_cast<uint32_t>(i - static_cast<uint64_t>(page) * n);
        mmc::dev::on_page_masks(h, page, n)[w] = 0u;
    }
    if(blockIdx.x == 0 && threadIdx.x == 0)
    {
        h.state->firstfreeblock = 0u;
        h.state->pagebasedMutex = 0u;
        h.state->firstFreePageBased = h.numpages - 1u;
        h.state->error_flags = 0u;
    }
}

/* Pass 1 of getAvailableSlotsHost (Scatter.hpp:1245-1285 over
 * getAvailaibleSlotsDeviceFunction, :1158-1219). Each block owns a contiguous
 * page range. slot < pagesize: per-page free chunks summed (u32, wrapping as
 * the reference's unsigned does). slot >= pagesize: run summaries folded in
 * page order. */
template<bool MULTI>
__global__ void __launch_bounds__(kScanThreads) mmc_slots_pass1(mmc_device_handle h, uint32_t slot,
                                                                SlotPartial* partials)
{
    const uint32_t np = h.numpages;
    const uint32_t per_block = (np + gridDim.x - 1u) / gridDim.x;
    const uint32_t b0 = min(blockIdx.x * per_block, np);
    const uint32_t b1 = min(b0 + per_block, np);
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = threadIdx.x >> 5;
    constexpr uint32_t nwarps = kScanThreads / 32u;
    if(!MULTI)
    {
        const uint32_t P = h.pagesize;
        const uint32_t maxchunksize = mmc::dev::umin(P, h.wastefactor * slot);
        const uint32_t slotChunk = mmc::dev::umax(slot, h.paddedMinChunkSize);
        const uint32_t capSlotChunk = mmc::dev::page_capacity(h, slotChunk);
        uint32_t sum = 0u;
        for(uint32_t pg = b0 + threadIdx.x; pg < b1; pg += kScanThreads)
            sum += mmc::dev::page_free_slots(h, __ldcg(&h.chunksize[pg]), __ldcg(&h.count[pg]), slot, maxchunksize,
                                             slotChunk, capSlotChunk);
        sum = __reduce_add_sync(0xFFFFFFFFu, sum);
        __shared__ uint32_t ws[nwarps];
        if(lane == 0)
            ws[warp] = sum;
        __syncthreads();
        if(threadIdx.x == 0)
        {
            uint32_t t = 0u;
            for(uint32_t w = 0; w < nwarps; ++w)
                t += ws[w];
            partials[blockIdx.x] = SlotPartial{0u, 0u, 0u, t};
        }
        return;
    }
    const uint32_t n = (slot + h.pagesize - 1u) / h.pagesize;
    /* each warp folds a contiguous sub-range in tiles of 32 pages */
    const uint32_t per_warp = (b1 - b0 + nwarps - 1u) / nwarps;
    const uint32_t w0 = min(b0 + warp * per_warp, b1);
    const uint32_t w1 = min(w0 + per_warp, b1);
    RunSum acc = mmc::dev::run_empty();
    for(uint32_t t0 = w0; t0 < w1; t0 += 32u)
    {
        const uint32_t pg = t0 + lane;
        RunSum s = pg < w1 ? mmc::dev::run_leaf(__ldcg(&h.chunksize[pg]) == 0u) : mmc::dev::run_empty();
#pragma unroll
        for(uint32_t off = 1u; off < 32u; off <<= 1)
        {
            const RunSum o = mmc::dev::shfl_runsum(0xFFFFFFFFu, s, static_cast<int>((lane + off) & 31u));
            if((lane & (2u * off - 1u)) == 0u && lane + off < 32u)
                s = mmc::dev::run_combine(s, o, n);
        }
        acc = mmc::dev::run_combine(acc, s, n); /* lane 0 holds the tile fold */
    }
    __shared__ RunSum wsum[nwarps];
    if(lane == 0)
        wsum[warp] = acc;
    __syncthreads();
    if(threadIdx.x == 0)
    {
        RunSum b = mmc::dev::run_empty();
        for(uint32_t w = 0; w < nwarps; ++w)
            b = mmc::dev::run_combine(b, wsum[w], n);
        partials[blockIdx.x] = SlotPartial{b.len, b.pre, b.suf, b.cnt};
    }
}

/* Pass 2: fold the block partials in order; write the unsigned result. */
__global__ void mmc_slots_pass2(const SlotPartial* partials, uint32_t nparts, uint32_t multi, uint32_t n,
                                unsigned* out)
{
    const uint32_t lane = threadIdx.x;
    const uint32_t per = (nparts + 31u) / 32u;
    const uint32_t a = min(lane * per, nparts);
    const uint32_t b = min(a + per, nparts);
    if(!multi)
    {
        uint32_t sum = 0u;
        for(uint32_t i = a; i < b; ++i)
            sum += partials[i].cnt;
        sum = __reduce_add_sync(0xFFFFFFFFu, sum);
        if(lane == 0)
            *out = sum;
        return;
    }
    RunSum s = mmc::dev::run_empty();
    for(uint32_t i = a; i < b; ++i)
    {
        const SlotPartial p = partials[i];
        s = mmc::dev::run_combine(s, RunSum{p.len, p.pre, p.suf, p.cnt}, n);
    }
#pragma unroll
    for(uint32_t off = 1u; off < 32u; off <<= 1)
    {
        const RunSum o = mmc::dev::shfl_runsum(0xFFFFFFFFu, s, static_cast<int>((lane + off) & 31u));
        if((lane & (2u * off - 1u)) == 0u && lane + off < 32u)
            s = mmc::dev::run_combine(s, o, n);
    }
    if(lane == 0)
        *out = mmc::dev::run_total(s, n);
}

/* Scratch of mmc_available_slots_noalloc: one scan partial per block. Every
 * GPU that loads the library holds it (32 KiB) until the process exits; in host
 * code the name is not a device address, so it is reached only through the
 * address cudaGetSymbolAddress returns for the current device. */
static __device__ __align__(256) SlotPartial g_noalloc_partials[MMC_NOALLOC_SCAN_BLOCKS_MAX];

namespace
{
    constexpr int kNoallocMaxDevices = 64;
    std::mutex g_noalloc_mutex;
    /* the array's device address per device ordinal, with the id of the
     * context it was looked up in: after a cudaDeviceReset, or for a caller
     * whose current context on that ordinal is another one, the ids differ
     * and the address is looked up again */
    struct NoallocAddr
    {
        unsigned long long ctx_id;
        SlotPartial* addr;
    };
    NoallocAddr g_noalloc_addr[kNoallocMaxDevices] = {};

    /* Unique id of the calling thread's current CUDA context (cuCtxGetId,
     * reached through the runtime's driver entry points so the library does
     * not link libcuda); 0 when there is none yet or the driver lacks it. */
    unsigned long long current_context_id()
    {
        using GetCurrent = CUresult (*)(CUcontext*);
        using GetId = CUresult (*)(CUcontext, unsigned long long*);
        static GetCurrent get_current = nullptr;
        static GetId get_id = nullptr;
        static bool looked_up = false;
        if(!looked_up)
        {
            looked_up = true;
            void* f = nullptr;
            cudaDriverEntryPointQueryResult q;
            if(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess
               && q == cudaDriverEntryPointSuccess)
                get_current = reinterpret_cast<GetCurrent>(f);
            f = nullptr;
            if(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess
               && q == cudaDriverEntryPointSuccess)
                get_id = reinterpret_cast<GetId>(f);
            cudaGetLastError();
        }
        CUcontext ctx = nullptr;
        unsigned long long id = 0ull;
        if(get_current == nullptr || get_id == nullptr || get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr
           || get_id(ctx, &id) != CUDA_SUCCESS)
            return 0ull;
        return id;
    }
} // namespace

/* ------------------------------------------------------------- host logic */

namespace
{
    bool is_pow2(uint64_t x) { return x != 0u && (x & (x - 1u)) == 0u; }

    mmc_status validate(const mmc_config* c)
    {
        if(c == nullptr)
            return fail(MMC_ERR_ARG, "config is null");
        if(c->pagesize < 256u || (c->pagesize % 16u) != 0u)
            return fail(MMC_ERR_CONFIG, "pagesize must be a multiple of 16 and at least 256");
        if(c->regionsize == 0u || c->wastefactor == 0u || c->accessblocksize == 0u)
            return fail(MMC_ERR_CONFIG, "regionsize, wastefactor and accessblocksize must be non-zero");
        if(c->dataAlignment > 1u && !is_pow2(c->dataAlignment))
            return fail(MMC_ERR_CONFIG, "dataAlignment must be a power of 2");
        if(c->distribution > MMC_DIST_XMALLOCSIMD)
            return fail(MMC_ERR_CONFIG, "unknown distribution policy");
        if(c->oom_policy > MMC_OOM_FLAG)
            return fail(MMC_ERR_CONFIG, "unknown OOM policy");
        return MMC_OK;
    }

    /* initDeviceFunction's layout arithmetic (Scatter.hpp:962-1019), on the host. */
    mmc_status compute_geometry(const mmc_config& c, const char* pool, size_t memsize, mmc_geometry* g)
    {
        const uint32_t P = c.pagesize;
        const uint32_t R = c.regionsize;
        uint32_t numregions = static_cast<uint32_t>(static_cast<uint64_t>(memsize)
                                                    / (static_cast<uint64_t>(R) * (12u + P) + 4u));
        uint32_t numpages = numregions * R;
        const uint64_t memorysize = static_cast<uint64_t>(numpages) * P;
        const uint64_t numblocks = memorysize / c.accessblocksize;
        if(numblocks == 0u)
            return fail(MMC_ERR_CONFIG, "heap smaller than one access block (the reference divides by zero here, "
                                        "Scatter.hpp:991-993)");
        const uint64_t memoryperblock = memorysize / numblocks;
        const uint64_t pagesperblock = memoryperblock / P;
        const uint64_t regionsperblock = pagesperblock / R;
        numregions = static_cast<uint32_t>(numblocks * regionsperblock);
        numpages = numregions * R;
        if(numpages == 0u)
            return fail(MMC_ERR_CONFIG, "access block smaller than one region");
        const uint64_t end = static_cast<uint64_t>(numpages) * P + 12ull * numpages + 4ull * numregions;
        if(end > memsize)
        {
            --numregions;
            numpages = std::min(numregions * R, numpages);
        }
        const uint32_t minChunk = (P - 128u) / 1024u;
        const uint32_t ht = (P - 8u) / 33u;
        const uint32_t minSeg = 32u * minChunk + 4u;
        const uint32_t onPage = minChunk > ht ? 0u : (P + (minSeg - 1u)) / minSeg;
        g->memsize = memsize;
        g->numpages = numpages;
        g->numregions = numregions;
        g->accessblocks = static_cast<uint32_t>(numblocks);
        g->pagesperblock = numpages / static_cast<uint32_t>(numblocks);
        g->maxOnPageMasks = std::min(32u, onPage);
        g->hierarchyThreshold = ht;
        g->ptes_offset = static_cast<uint64_t>(numpages) * P;
        g->regions_offset = g->ptes_offset + 12ull * numpages;
        (void) pool;
        return MMC_OK;
    }

    void fill_handle(mmc_heap* h)
    {
        mmc_device_handle& d = h->handle;
        const mmc_config& c = h->cfg;
        const mmc_geometry& g = h->geom;
        d.state = h->state;
        d.pages = h->pool;
        d.chunksize = reinterpret_cast<uint32_t*>(h->pool + g.ptes_offset);
        d.count = d.chunksize + g.numpages;
        d.bitmask = d.count + g.numpages;
        d.regions = reinterpret_cast<uint32_t*>(h->pool + g.regions_offset);
        d.freemap = h->freemap;
        d.numpages = g.numpages;
        d.numregions = g.numregions;
        d.accessblocks = g.accessblocks;
        d.pagesperblock = g.pagesperblock;
        d.pagesize = c.pagesize;
        d.regionsize = c.regionsize;
        d.wastefactor = c.wastefactor;
        d.resetfreedpages = c.resetfreedpages ? 1u : 0u;
        d.hashingK = c.hashingK;
        d.hashingDistMP = c.hashingDistMP;
        d.hashingDistWP = c.hashingDistWP;
        d.hashingDistWPRel = c.hashingDistWPRel;
        d.dataAlignment = c.dataAlignment;
        d.distribution = c.distribution;
        d.oom_policy = c.oom_policy;
        d.reference_quirks = c.reference_quirks ? 1u : 0u;
        d.hierarchyThreshold = g.hierarchyThreshold;
        d.minChunkSize = (c.pagesize - 128u) / 1024u;
        d.paddedMinChunkSize = mmc::dev::apply_padding(c.dataAlignment, d.minChunkSize);
        d.maxOnPageMasks = g.maxOnPageMasks;
    }

    /* Shrink::alignPool (Shrink.hpp:109-130), including its size arithmetic. */
    void align_pool(uint32_t align, char** pool, size_t* memsize)
    {
        if(align <= 1u)
            return;
        const uintptr_t status = reinterpret_cast<uintptr_t>(*pool) & (align - 1u);
        if(status != 0u)
        {
            *pool += align - status;
            *memsize -= align + status;
        }
    }

    /* words of the free-page bitmap: one bit per page and a clear bit for page
     * numpages, rounded up to whole 16-byte groups (the search reads four
     * words at a time) and one spare group */
    size_t freemap_words_for(uint32_t numpages) { return ((static_cast<size_t>(numpages) / 32u + 1u + 3u) & ~size_t{3}) + 4u; }

    mmc_status init_heap(mmc_heap* h, cudaStream_t s)
    {
        mmc_status st = compute_geometry(h->cfg, h->pool, h->memsize, &h->geom);
        if(st != MMC_OK)
            return st;
        const size_t fm_words = freemap_words_for(h->geom.numpages);
        if(fm_words > h->freemap_words)
        {
            if(h->freemap)
                cudaFree(h->freemap);
            h->freemap = nullptr;
            h->freemap_words = 0;
            if(cudaMalloc(&h->freemap, fm_words * 4u) != cudaSuccess)
            {
                cudaGetLastError();
                h->freemap = nullptr;
                return fail(MMC_ERR_OOM, "cudaMalloc of the free-page bitmap failed");
            }
            h->freemap_words = fm_words;
        }
        fill_handle(h);
        const mmc_geometry& g = h->geom;
        st = cuda_check(cudaMemsetAsync(h->pool + g.ptes_offset, 0, 12ull * g.numpages + 4ull * g.numregions, s),
                        "zero page table");
        if(st == MMC_OK)
            st = cuda_check(cudaMemsetAsync(h->state, 0, sizeof(mmc_heap_state), s), "zero heap header");
        if(st != MMC_OK)
            return st;
        const uint64_t words = static_cast<uint64_t>(g.numpages) * g.maxOnPageMasks;
        const unsigned grid = static_cast<unsigned>(
            std::max<uint64_t>(1u, std::min<uint64_t>((words + 255u) / 256u, scan_grid(h->device) * 8u)));
        mmc_init_kernel<<<grid, 256, 0, s>>>(h->handle, static_cast<uint32_t>(h->freemap_words));
        return cuda_check(cudaGetLastError(), "heap init kernel");
    }

    mmc_status create_common(const mmc_config* cfg, void* pool, size_t bytes, bool owns, int device, void* stream,
                             mmc_heap** out)
    {
        if(out == nullptr)
            return fail(MMC_ERR_ARG, "out is null");
        *out = nullptr;
        mmc_status st = validate(cfg);
        if(st != MMC_OK)
            return st;
        if(owns)
        {
            /* cudaMalloc returns 256-byte aligned memory, so Shrink::alignPool
             * leaves the size alone: the geometry can be checked before any
             * device work */
            mmc_geometry g;
            st = compute_geometry(*cfg, nullptr, bytes, &g);
            if(st != MMC_OK)
                return st;
        }
        st = cuda_check(cudaSetDevice(device), "cudaSetDevice");
        if(st != MMC_OK)
            return st;
        mmc_heap* h = new(std::nothrow) mmc_heap();
        if(h == nullptr)
            return fail(MMC_ERR_OOM, "host allocation failed");
        h->cfg = *cfg;
        h->device = device;
        h->scan_blocks = scan_grid(device);
        cudaStream_t s = as_stream(stream);
        if(owns)
        {
            if(bytes == 0u)
            {
                delete h;
                return fail(MMC_ERR_CONFIG, "heap size is zero");
            }
            if(cudaMalloc(&pool, bytes) != cudaSuccess)
            {
                cudaGetLastError();
                delete h;
                return fail(MMC_ERR_OOM, "cudaMalloc of the pool failed (" + std::to_string(bytes) + " bytes)");
            }
        }
        else if(pool == nullptr)
        {
            delete h;
            return fail(MMC_ERR_ARG, "Scatter policy cannot use nullptr for non-empty memory pools "
                                     "(Scatter.hpp:1065-1071)");
        }
        h->pool_raw = pool;
        h->pool_raw_bytes = bytes;
        h->owns_pool = owns;
        h->pool = static_cast<char*>(pool);
        h->memsize = bytes;
        align_pool(cfg->dataAlignment, &h->pool, &h->memsize);
        const size_t devbytes = sizeof(mmc_heap_state) + sizeof(SlotPartial) * kMaxScanBlocks + 128u;
        if(cudaMalloc(&h->devblock, devbytes) != cudaSuccess
           || cudaMallocHost(reinterpret_cast<void**>(&h->host_result), sizeof(unsigned)) != cudaSuccess)
        {
            cudaGetLastError();
            if(h->devblock)
                cudaFree(h->devblock);
            if(owns)
                cudaFree(pool);
            delete h;
            return fail(MMC_ERR_OOM, "cudaMalloc of the heap header failed");
        }
        h->state = reinterpret_cast<mmc_heap_state*>(h->devblock);
        h->partials = reinterpret_cast<SlotPartial*>(h->devblock + sizeof(mmc_heap_state));
        h->result_word = reinterpret_cast<unsigned*>(h->devblock + sizeof(mmc_heap_state)
                                                     + sizeof(SlotPartial) * kMaxScanBlocks);
        st = init_heap(h, s);
        if(st != MMC_OK)
        {
            mmc_heap_destroy(h);
            return st;
        }
        *out = h;
        return MMC_OK;
    }
} // namespace

namespace mmc
{
    namespace host
    {
        mmc_status launch_available_slots(mmc_heap* heap, uint32_t slot, cudaStream_t s, unsigned* result_dev)
        {
            const bool multi = slot >= heap->cfg.pagesize;
            const unsigned grid = heap->scan_blocks;
            if(multi)
                mmc_slots_pass1<true><<<grid, kScanThreads, 0, s>>>(heap->handle, slot, heap->partials);
            else
                mmc_slots_pass1<false><<<grid, kScanThreads, 0, s>>>(heap->handle, slot, heap->partials);
            const uint32_t n = (slot + heap->cfg.pagesize - 1u) / heap->cfg.pagesize;
            mmc_slots_pass2<<<1, 32, 0, s>>>(heap->partials, grid, multi ? 1u : 0u, n, result_dev);
            return cuda_check(cudaGetLastError(), "available slots kernels");
        }
    } // namespace host
} // namespace mmc

/* ---------------------------------------------------------------- C ABI */

extern "C" {

void mmc_config_default(mmc_config* c)
{
    if(c == nullptr)
        return;
    std::memset(c, 0, sizeof(*c));
    c->pagesize = 4096u;
    c->regionsize = 16u;
    c->wastefactor = 2u;
    c->resetfreedpages = 0u;
    c->accessblocksize = 2ull * 1024ull * 1024ull * 1024ull;
    c->hashingK = 38183u;
    c->hashingDistMP = 17497u;
    c->hashingDistWP = 1u;
    c->hashingDistWPRel = 1u;
    c->dataAlignment = 16u;
    c->distribution = MMC_DIST_XMALLOCSIMD;
    c->oom_policy = MMC_OOM_RETURNNULL;
    c->reference_quirks = 1u;
}

mmc_status mmc_heap_create(const mmc_config* cfg, size_t bytes, int device, void* stream, mmc_heap** out)
{
    return create_common(cfg, nullptr, bytes, true, device, stream, out);
}

mmc_status mmc_heap_create_on_pool(const mmc_config* cfg, void* pool, size_t bytes, int device, void* stream,
                                   mmc_heap** out)
{
    mmc::host::NvtxRange nvtx_range("mmc_heap_create");
    return create_common(cfg, pool, bytes, false, device, stream, out);
}

mmc_status mmc_heap_destroy(mmc_heap* h)
{
    if(h == nullptr)
        return MMC_OK;
    cudaSetDevice(h->device);
    cudaDeviceSynchronize();
    if(h->owns_pool && h->pool_raw)
        cudaFree(h->pool_raw);
    if(h->devblock)
        cudaFree(h->devblock);
    if(h->freemap)
        cudaFree(h->freemap);
    if(h->host_result)
        cudaFreeHost(h->host_result);
    delete h;
    return MMC_OK;
}

mmc_status mmc_heap_destructive_resize(mmc_heap* h, size_t bytes, void* stream)
{
    if(h == nullptr)
        return fail(MMC_ERR_ARG, "heap is null");
    if(!h->owns_pool)
        return fail(MMC_ERR_ARG, "destructive resize needs a heap that owns its pool");
    cudaSetDevice(h->device);
    cudaStream_t s = as_stream(stream);
    mmc_status st = cuda_check(cudaStreamSynchronize(s), "synchronise before resize");
    if(st != MMC_OK)
        return st;
    cudaFree(h->pool_raw);
    h->pool_raw = nullptr;
    void* pool = nullptr;
    if(bytes == 0u || cudaMalloc(&pool, bytes) != cudaSuccess)
    {
        cudaGetLastError();
        return fail(MMC_ERR_OOM, "cudaMalloc of the resized pool failed");
    }
    h->pool_raw = pool;
    h->pool_raw_bytes = bytes;
    h->pool = static_cast<char*>(pool);
    h->memsize = bytes;
    align_pool(h->cfg.dataAlignment, &h->pool, &h->memsize);
    return init_heap(h, s);
}

mmc_status mmc_heap_device_handle(const mmc_heap* h, mmc_device_handle* out)
{
    if(h == nullptr || out == nullptr)
        return fail(MMC_ERR_ARG, "null argument");
    *out = h->handle;
    return MMC_OK;
}

mmc_status mmc_heap_locations(const mmc_heap* h, void** pool, size_t* size)
{
    if(h == nullptr)
        return fail(MMC_ERR_ARG, "heap is null");
    if(pool)
        *pool = h->pool;
    if(size)
        *size = h->memsize;
    return MMC_OK;
}

mmc_status mmc_heap_geometry(const mmc_heap* h, mmc_geometry* out)
{
    if(h == nullptr || out == nullptr)
        return fail(MMC_ERR_ARG, "null argument");
    *out = h->geom;
    return MMC_OK;
}

mmc_status mmc_heap_info(const mmc_heap* h, char* buf, size_t len)
{
    if(h == nullptr || buf == nullptr || len == 0u)
        return fail(MMC_ERR_ARG, "null argument");
    const mmc_config& c = h->cfg;
    std::ostringstream ss;
    ss << "CreationPolicy:      Scatter[pagesize=" << c.pagesize << ",accessblocksize=" << c.accessblocksize
       << ",regionsize=" << c.regionsize << ",wastefactor=" << c.wastefactor
       << ",resetfreedpages=" << (c.resetfreedpages ? 1 : 0) << ",minChunkSize=" << h->handle.minChunkSize
       << ",HierarchyThreshold=" << h->handle.hierarchyThreshold << ",hashingK=" << c.hashingK
       << ",hashingDistMP=" << c.hashingDistMP << ",hashingDistWP=" << c.hashingDistWP
       << ",hashingDistWPRel=" << c.hashingDistWPRel << "]\n";
    ss << "DistributionPolicy:  "
       << (c.distribution == MMC_DIST_XMALLOCSIMD ? "XMallocSIMD[" + std::to_string(c.pagesize) + "]"
                                                  : std::string("Noop"))
       << "\n";
    ss << "OOMPolicy:           " << (c.oom_policy == MMC_OOM_RETURNNULL ? "ReturnNull" : "BadAllocFlag") << "\n";
    ss << "ReservePoolPolicy:   " << (h->owns_pool ? "AlpakaBuf" : "ExternalPool") << "\n";
    ss << "AlignmentPolicy:     "
       << (c.dataAlignment > 1u ? "Shrink[" + std::to_string(c.dataAlignment) + "]" : std::string("Noop")) << "\n";
    const std::string s = ss.str();
    const size_t n = std::min(len - 1u, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = '\0';
    return MMC_OK;
}

mmc_status mmc_available_slots_async(mmc_heap* h, size_t slot_size, void* stream, unsigned* out_dev)
{
    mmc::host::NvtxRange nvtx_range("mmc_available_slots");
    if(h == nullptr || out_dev == nullptr)
        return fail(MMC_ERR_ARG, "null argument");
    const uint32_t slot = mmc::dev::apply_padding(h->cfg.dataAlignment, static_cast<uint32_t>(slot_size));
    return launch_available_slots(h, slot, as_stream(stream), out_dev);
}

mmc_status mmc_available_slots_noalloc(const mmc_device_handle* handle, size_t slot_size, unsigned scan_blocks,
                                       void* stream, unsigned* out_dev)
{
    if(handle == nullptr || out_dev == nullptr)
        return fail(MMC_ERR_ARG, "null argument");
    int dev = 0;
    mmc_status st = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if(st != MMC_OK)
        return st;
    if(dev < 0 || dev >= kNoallocMaxDevices)
        return fail(MMC_ERR_ARG, "device ordinal beyond the no-alloc entry point's table");
    if(scan_blocks == 0u)
        scan_blocks = scan_grid(dev);
    if(scan_blocks > MMC_NOALLOC_SCAN_BLOCKS_MAX)
        return fail(MMC_ERR_ARG, "scan_blocks " + std::to_string(scan_blocks) + " exceeds the static scratch of "
                                     + std::to_string(MMC_NOALLOC_SCAN_BLOCKS_MAX) + " partials");
    SlotPartial* partials = nullptr;
    {
        /* set-up, once per device and context, with that device current */
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        NoallocAddr& a = g_noalloc_addr[dev];
        const unsigned long long ctx = current_context_id();
        if(a.addr == nullptr || ctx == 0ull || a.ctx_id != ctx)
        {
            void* p = nullptr;
            st = cuda_check(cudaGetSymbolAddress(&p, g_noalloc_partials), "cudaGetSymbolAddress");
            if(st != MMC_OK)
                return st;
            /* the lookup makes the device's context current if it was not yet */
            a.ctx_id = ctx != 0ull ? ctx : current_context_id();
            a.addr = static_cast<SlotPartial*>(p);
        }
        partials = a.addr;
    }
    const uint32_t slot = mmc::dev::apply_padding(handle->dataAlignment, static_cast<uint32_t>(slot_size));
    const bool multi = slot >= handle->pagesize;
    cudaStream_t s = as_stream(stream);
    if(multi)
        mmc_slots_pass1<true><<<scan_blocks, kScanThreads, 0, s>>>(*handle, slot, partials);
    else
        mmc_slots_pass1<false><<<scan_blocks, kScanThreads, 0, s>>>(*handle, slot, partials);
    const uint32_t n = (slot + handle->pagesize - 1u) / handle->pagesize;
    mmc_slots_pass2<<<1, 32, 0, s>>>(partials, scan_blocks, multi ? 1u : 0u, n, out_dev);
    return cuda_check(cudaGetLastError(), "no-alloc slot count kernels");
}

mmc_status mmc_available_slots(mmc_heap* h, size_t slot_size, void* stream, unsigned* out)
{
    if(h == nullptr || out == nullptr)
        return fail(MMC_ERR_ARG, "null argument");
    cudaSetDevice(h->device);
    cudaStream_t s = as_stream(stream);
    mmc_status st = mmc_available_slots_async(h, slot_size, stream, h->result_word);
    if(st != MMC_OK)
        return st;
    st = cuda_check(cudaMemcpyAsync(h->host_result, h->result_word, sizeof(unsigned), cudaMemcpyDeviceToHost, s),
                    "copy slot count");
    if(st != MMC_OK)
        return st;
    st = cuda_check(cudaStreamSynchronize(s), "wait for slot count");
    if(st != MMC_OK)
        return st;
    *out = *h->host_result;
    return MMC_OK;
}

mmc_status mmc_heap_error(mmc_heap* h, void* stream, uint32_t* flags, int clear)
{
    if(h == nullptr || flags == nullptr)
        return fail(MMC_ERR_ARG, "null argument");
    cudaStream_t s = as_stream(stream);
    mmc_status st = cuda_check(cudaMemcpyAsync(h->host_result, &h->state->error_flags, sizeof(uint32_t),
                                               cudaMemcpyDeviceToHost, s),
                               "copy error word");
    if(st == MMC_OK)
        st = cuda_check(cudaStreamSynchronize(s), "wait for error word");
    if(st != MMC_OK)
        return st;
    *flags = *h->host_result;
    if(clear)
    {
        st = cuda_check(cudaMemsetAsync(&h->state->error_flags, 0, sizeof(uint32_t), s), "clear error word");
        if(st == MMC_OK)
            st = cuda_check(cudaStreamSynchronize(s), "wait for clear");
    }
    return st;
}

mmc_status mmc_heap_stats(mmc_heap* h, void* stream, unsigned long long* out, int clear)
{
    if(h == nullptr || out == nullptr)
        return fail(MMC_ERR_ARG, "null argument");
    cudaStream_t s = as_stream(stream);
    mmc_status st = cuda_check(cudaStreamSynchronize(s), "synchronise before stats");
    if(st == MMC_OK)
        st = cuda_check(cudaMemcpy(out, h->state->stats, sizeof(unsigned long long) * MMC_STAT_COUNT,
                                   cudaMemcpyDeviceToHost),
                        "copy stats");
    if(st == MMC_OK && clear)
        st = cuda_check(cudaMemset(h->state->stats, 0, sizeof(unsigned long long) * MMC_STAT_COUNT), "clear stats");
    return st;
}

mmc_status mmc_snapshot_freemap(mmc_heap* h, void* stream, uint32_t* words)
{
    if(h == nullptr || words == nullptr)
        return fail(MMC_ERR_ARG, "null argument");
    cudaStream_t s = as_stream(stream);
    const size_t n = (static_cast<size_t>(h->geom.numpages) + 31u) / 32u;
    mmc_status st = cuda_check(cudaStreamSynchronize(s), "synchronise before freemap snapshot");
    if(st == MMC_OK)
        st = cuda_check(cudaMemcpy(words, h->freemap, n * 4u, cudaMemcpyDeviceToHost), "copy freemap");
    return st;
}

mmc_status mmc_snapshot_metadata(mmc_heap* h, void* stream, uint32_t* ptes3, uint32_t* regions, uint32_t* masks,
                                 uint32_t* header3)
{
    if(h == nullptr)
        return fail(MMC_ERR_ARG, "heap is null");
    cudaSetDevice(h->device);
    cudaStream_t s = as_stream(stream);
    mmc_status st = cuda_check(cudaStreamSynchronize(s), "synchronise before snapshot");
    if(st != MMC_OK)
        return st;
    const mmc_geometry& g = h->geom;
    const mmc_device_handle& d = h->handle;
    if(ptes3)
    {
        uint32_t* tmp = new(std::nothrow) uint32_t[3ull * g.numpages];
        if(tmp == nullptr)
            return fail(MMC_ERR_OOM, "host allocation failed");
        st = cuda_check(cudaMemcpy(tmp, d.chunksize, 12ull * g.numpages, cudaMemcpyDeviceToHost), "copy ptes");
        if(st == MMC_OK)
            for(uint64_t i = 0; i < g.numpages; ++i)
            {
                ptes3[3 * i + 0] = tmp[i];
                ptes3[3 * i + 1] = tmp[g.numpages + i];
                ptes3[3 * i + 2] = tmp[2ull * g.numpages + i];
            }
        delete[] tmp;
        if(st != MMC_OK)
            return st;
    }
    if(regions)
    {
        st = cuda_check(cudaMemcpy(regions, d.regions, 4ull * g.numregions, cudaMemcpyDeviceToHost), "copy regions");
        if(st != MMC_OK)
            return st;
    }
    if(masks && g.maxOnPageMasks > 0u)
    {
        const size_t w = 4u * g.maxOnPageMasks;
        st = cuda_check(cudaMemcpy2D(masks, w, h->pool + h->cfg.pagesize - w, h->cfg.pagesize, w, g.numpages,
                                     cudaMemcpyDeviceToHost),
                        "copy on-page masks");
        if(st != MMC_OK)
            return st;
    }
    if(header3)
    {
        mmc_heap_state hs;
        st = cuda_check(cudaMemcpy(&hs, h->state, sizeof(hs), cudaMemcpyDeviceToHost), "copy header");
        if(st != MMC_OK)
            return st;
        header3[0] = hs.firstFreePageBased;
        header3[1] = hs.firstfreeblock;
        header3[2] = hs.pagebasedMutex;
    }
    return MMC_OK;
}

const char* mmc_last_error(void) { return g_last_error.c_str(); }

} /* extern "C" */

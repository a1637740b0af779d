/* serve.cu — a continuous-batching request server on a device-resident heap.
 *
 * A request is a sequence of 2-byte elements that grows to a final length; it
 * holds one 16 KiB chunk (malloc'd from the heap) per 256 elements, writes its
 * elements (a seeded function of request and index) into them, and when it
 * reaches its final length reads them all back into a checksum and frees its
 * chunks. All request state lives on the device in a slot table.
 *
 * One tick = one launch (replayed from a captured CUDA graph in the batched
 * form): it applies the host's admissions and slot releases for this tick,
 * grows every live request by `step` elements (one warp per slot), completes
 * the requests that reach their length, and refreshes the free-slot count of
 * 16 KiB chunks that the host admits against. The per-request form launches
 * one grow kernel per live request instead.
 *
 * Host and device meet in mapped pinned memory: the kernels read the tick's
 * commands where the host wrote them, write every slot they change through to
 * the host's copy of the slot table, and the free-chunk count lands in host
 * memory, so a tick has no copy steps (on GB300 the device reaches host
 * memory over NVLink-C2C).
 *
 * Pipelined ticks alternate between two buffers, each with its own command
 * queue and its own published results (the requests that completed in the
 * tick, with their checksums; the chunks the live requests will yet take; the
 * free-chunk count). While tick i runs on one buffer, the host reads what tick
 * i - 1 published in the other and writes tick i + 1's commands there, so host
 * and device work overlap and the host never reads what a running tick writes.
 */
#include "mmc_internal.h"

#include <cstring>
#include <new>
#include <string>
#include <vector>

using namespace mmc::host;
namespace dv = mmc::dev;

namespace
{
    constexpr uint32_t kChunkBytes = 16384;
    constexpr uint32_t kElemsPerChunk = 256;
    static_assert(kElemsPerChunk * 2u == 32u * 16u, "a chunk's elements are one 16-byte load per lane of a warp");

    __host__ __device__ __forceinline__ uint64_t mix64(uint64_t seed, uint64_t a, uint64_t b)
    {
        uint64_t z = seed + a * 0x9E3779B97F4A7C15ull + b * 0xD1B54A32D192ED03ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
} // namespace

struct mmc_server
{
    mmc_heap* heap;
    mmc_device_handle handle;
    int device;
    uint32_t slots;
    uint32_t max_chunks;
    uint32_t step;
    uint32_t queue_cap;
    mmc_serve_slot* d_slots;   /* slot table */
    void** d_chunks;           /* slots x max_chunks chunk pointers */
    mmc_serve_cmd* h_queue;    /* this tick's admissions / releases (mapped pinned) */
    uint32_t* h_queue_len;     /* mapped pinned */
    mmc_serve_slot* h_slots;   /* the host's copy of the slot table, written through by the kernels */
    unsigned* h_free;          /* free 16 KiB slots after the tick (mapped pinned) */
    /* device addresses of the mapped pinned buffers above */
    const mmc_serve_cmd* m_queue;
    const uint32_t* m_queue_len;
    mmc_serve_slot* m_slots;
    unsigned* m_free;
    /* the fused free-slot count: one sum per scan block and the count of
     * blocks that have added theirs (zero between ticks) */
    uint32_t count_blocks;
    uint32_t* d_count_partials;
    uint32_t* d_count_arrived;
    cudaStream_t stream;
    cudaGraphExec_t exec;
    cudaGraph_t graph;
    /* pipelined ticks: per buffer a command queue and the tick's published
     * results (mapped pinned, h_* the host's addresses and m_* the device's),
     * the completion list and counters the tick builds in device memory, and
     * the captured tick graph */
    struct Pipe
    {
        mmc_serve_cmd* h_queue;
        uint32_t* h_queue_len;
        const mmc_serve_cmd* m_queue;
        const uint32_t* m_queue_len;
        mmc_serve_done* h_done;
        uint32_t* h_done_len;
        unsigned long long* h_remaining;
        unsigned* h_free;
        mmc_serve_done* m_done;
        uint32_t* m_done_len;
        unsigned long long* m_remaining;
        unsigned* m_free;
        mmc_serve_done* d_done;
        unsigned long long* d_counts; /* [0]: completions, [1]: chunks still to take */
        cudaGraph_t graph;
        cudaGraphExec_t exec;
        cudaEvent_t finished; /* recorded after each launch of this buffer's tick */
    } pipe[2];
};

/* Apply admissions (cmd.kind 1) and releases (cmd.kind 2), read from the
 * host's queue; each changed slot is also written to the host's table. The
 * queue lives in host-written memory, so nothing in it is trusted: a length
 * beyond the queue's capacity is cut to it, and a command naming a slot
 * beyond the table, an unknown kind or an admission longer than a slot's
 * chunks hold (max_len elements) is skipped; either sets MMC_DEVERR_BADCMD in
 * the heap's error word. */
__global__ void mmc_serve_apply(mmc_serve_slot* slots, mmc_serve_slot* mirror, const mmc_serve_cmd* q,
                                const uint32_t* qlen, uint32_t queue_cap, uint32_t nslots, uint32_t max_len,
                                uint32_t* error_flags)
{
    uint32_t n = *qlen;
    if(n > queue_cap)
    {
        if(blockIdx.x == 0u && threadIdx.x == 0u)
            atomicOr(error_flags, MMC_DEVERR_BADCMD);
        n = queue_cap;
    }
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const mmc_serve_cmd c = q[i];
        if(c.slot >= nslots || (c.kind != 1u && c.kind != 2u) || (c.kind == 1u && c.final_len > max_len))
        {
            atomicOr(error_flags, MMC_DEVERR_BADCMD);
            continue;
        }
        mmc_serve_slot& s = slots[c.slot];
        if(c.kind == 1u)
        {
            s.id = c.id;
            s.final_len = c.final_len;
            s.len = 0u;
            s.nchunks = 0u;
            s.seed = c.seed;
            s.failed = 0u;
            s.checksum = 0ull;
            s.state = MMC_SERVE_LIVE;
        }
        else if(c.kind == 2u)
            s.state = MMC_SERVE_FREE;
        mirror[c.slot] = s;
    }
}

/* Grow one live request by `step` elements (one warp), completing it at its length. */
template<class Ids>
__device__ __forceinline__ void grow_request(const mmc_device_handle& h, mmc_serve_slot& s, void** chunks,
                                             uint32_t max_chunks, uint32_t step)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t len = s.len;
    const uint32_t end = min(len + step, s.final_len);
    uint32_t failed = 0u;
    /* chunks this step needs: one per 256-element boundary crossed */
    const uint32_t first_chunk = (len + kElemsPerChunk - 1u) / kElemsPerChunk;
    const uint32_t last_chunk = (end + kElemsPerChunk - 1u) / kElemsPerChunk; /* exclusive */
    for(uint32_t c = first_chunk + lane; c < last_chunk && c < max_chunks; c += 32u)
    {
        void* p = dv::malloc<Ids>(h, kChunkBytes);
        chunks[c] = p;
        failed += p == nullptr;
    }
    failed = __reduce_add_sync(0xFFFFFFFFu, failed);
    __syncwarp();
    if(failed == 0u)
    {
        for(uint32_t e = len + lane; e < end; e += 32u)
        {
            uint16_t* chunk = static_cast<uint16_t*>(chunks[e / kElemsPerChunk]);
            chunk[e % kElemsPerChunk] = static_cast<uint16_t>(mix64(s.seed, e, 0x5E7ull));
        }
    }
    else
    {
        /* give back what this step took; the request retries next tick */
        for(uint32_t c = first_chunk + lane; c < last_chunk && c < max_chunks; c += 32u)
            if(chunks[c])
                dv::free<Ids>(h, chunks[c]);
    }
    __syncwarp();
    if(lane == 0u)
    {
        if(failed)
            s.failed += 1u;
        else
        {
            s.len = end;
            s.nchunks = last_chunk;
        }
    }
    __syncwarp();
    if(failed == 0u && end == s.final_len)
    {
        /* complete: read every element back, checksum, free the chunks. A
         * chunk's 256 elements are 512 contiguous bytes (at the chunk's
         * 16-byte aligned start), one 16-byte load per lane: the warp reads a
         * chunk per instruction, four chunks in flight, instead of 64 bytes
         * per instruction element by element. Bytes past the request's last
         * element lie inside its last chunk and are not summed. */
        unsigned long long sum = 0ull;
        const uint32_t nch = (end + kElemsPerChunk - 1u) / kElemsPerChunk;
#pragma unroll 4
        for(uint32_t c = 0; c < nch; ++c)
        {
            const uint4 v = reinterpret_cast<const uint4*>(chunks[c])[lane];
            const uint32_t w[4] = {v.x, v.y, v.z, v.w};
            const uint32_t e0 = c * kElemsPerChunk + lane * 8u;
#pragma unroll
            for(uint32_t k = 0; k < 8u; ++k)
            {
                const uint32_t e = e0 + k;
                const uint32_t x = (w[k / 2u] >> (16u * (k & 1u))) & 0xFFFFu;
                if(e < end)
                    sum += static_cast<unsigned long long>(x) * (e + 1ull);
            }
        }
        for(int off = 16; off > 0; off >>= 1)
            sum += __shfl_down_sync(0xFFFFFFFFu, sum, off);
        __syncwarp();
        for(uint32_t c = lane; c < last_chunk; c += 32u)
            dv::free<Ids>(h, chunks[c]);
        if(lane == 0u)
        {
            s.checksum = sum;
            s.state = MMC_SERVE_DONE;
        }
    }
}

/* Batched tick: one warp per slot; each grown slot is written to the host's
 * table. With `done` (pipelined ticks), a request that completes here is also
 * appended to the completion list, and each request still live adds the chunks
 * it will yet take to counts[1] (counts[0] is the list's length). */
template<class Ids>
__global__ void __launch_bounds__(256) mmc_serve_tick_kernel(mmc_device_handle h, mmc_serve_slot* slots,
                                                             mmc_serve_slot* mirror, void** chunks, uint32_t nslots,
                                                             uint32_t max_chunks, uint32_t step,
                                                             mmc_serve_done* done, unsigned long long* counts)
{
    const uint32_t warps = gridDim.x * (blockDim.x / 32u);
    for(uint32_t w = blockIdx.x * (blockDim.x / 32u) + threadIdx.x / 32u; w < nslots; w += warps)
    {
        if(slots[w].state != MMC_SERVE_LIVE)
            continue;
        grow_request<Ids>(h, slots[w], chunks + static_cast<uint64_t>(w) * max_chunks, max_chunks, step);
        __syncwarp();
        if((threadIdx.x & 31u) == 0u)
        {
            const mmc_serve_slot sw = slots[w];
            mirror[w] = sw;
            if(done != nullptr)
            {
                if(sw.state == MMC_SERVE_DONE)
                {
                    const unsigned long long i = atomicAdd(&counts[0], 1ull);
                    done[i] = mmc_serve_done{w, 0u, sw.checksum};
                }
                else
                {
                    const uint32_t need = (sw.final_len + kElemsPerChunk - 1u) / kElemsPerChunk;
                    atomicAdd(&counts[1], static_cast<unsigned long long>(need - sw.nchunks));
                }
            }
        }
    }
}

/* End of a pipelined tick: publish its completion list and counters to the
 * host (mapped memory) and zero the counters for the tick after next. One block. */
__global__ void mmc_serve_publish(const mmc_serve_done* done, unsigned long long* counts, mmc_serve_done* out,
                                  uint32_t* out_len, unsigned long long* out_remaining)
{
    const uint32_t n = static_cast<uint32_t>(counts[0]);
    for(uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        out[i] = done[i];
    __syncthreads();
    if(threadIdx.x == 0)
    {
        *out_len = n;
        *out_remaining = counts[1];
        counts[0] = 0ull;
        counts[1] = 0ull;
    }
}

/* The tick's free-slot count, getAvailableSlots(slot) for a slot below the
 * page size (the single-page branch, Scatter.hpp:1164-1193, summed over the
 * pages as mmc_slots_pass1/2 sum it), and for a pipelined tick the
 * publication of its results (mmc_serve_publish), in one kernel: each block
 * sums the free slots of its page range, and the last block to add its sum
 * (a device-scope arrival count, which that block sets back to zero for the
 * next tick) totals the block sums, writes the count and publishes. It saves
 * a tick two kernel boundaries over {pass 1, pass 2, publish}. No block waits
 * for another. */
constexpr uint32_t kCountThreads = 256;

template<bool PUBLISH>
__global__ void __launch_bounds__(kCountThreads)
    mmc_serve_count(mmc_device_handle h, uint32_t slot, uint32_t* partials, uint32_t* arrived, unsigned* out_free,
                    const mmc_serve_done* done, unsigned long long* counts, mmc_serve_done* out, uint32_t* out_len,
                    unsigned long long* out_remaining)
{
    constexpr uint32_t nwarps = kCountThreads / 32u;
    const uint32_t np = h.numpages;
    const uint32_t per_block = (np + gridDim.x - 1u) / gridDim.x;
    const uint32_t b0 = min(blockIdx.x * per_block, np);
    const uint32_t b1 = min(b0 + per_block, np);
    const uint32_t maxchunksize = dv::umin(h.pagesize, h.wastefactor * slot);
    const uint32_t slotChunk = dv::umax(slot, h.paddedMinChunkSize);
    const uint32_t capSlotChunk = dv::page_capacity(h, slotChunk);
    uint32_t sum = 0u;
    for(uint32_t pg = b0 + threadIdx.x; pg < b1; pg += kCountThreads)
        sum += dv::page_free_slots(h, __ldcg(&h.chunksize[pg]), __ldcg(&h.count[pg]), slot, maxchunksize, slotChunk,
                                   capSlotChunk);
    __shared__ uint32_t ws[nwarps];
    __shared__ bool last;
    sum = __reduce_add_sync(0xFFFFFFFFu, sum);
    if((threadIdx.x & 31u) == 0u)
        ws[threadIdx.x >> 5] = sum;
    __syncthreads();
    if(threadIdx.x == 0u)
    {
        uint32_t t = 0u;
        for(uint32_t w = 0; w < nwarps; ++w)
            t += ws[w];
        partials[blockIdx.x] = t;
        __threadfence(); /* the block's sum is visible before its arrival is */
        last = atomicAdd(arrived, 1u) == gridDim.x - 1u;
    }
    __syncthreads();
    if(!last)
        return;
    __threadfence(); /* the other blocks' sums are read after their arrivals */
    uint32_t t = 0u;
    for(uint32_t i = threadIdx.x; i < gridDim.x; i += kCountThreads)
        t += __ldcg(&partials[i]);
    t = __reduce_add_sync(0xFFFFFFFFu, t);
    __syncthreads();
    if((threadIdx.x & 31u) == 0u)
        ws[threadIdx.x >> 5] = t;
    __syncthreads();
    if(threadIdx.x == 0u)
    {
        uint32_t total = 0u;
        for(uint32_t w = 0; w < nwarps; ++w)
            total += ws[w];
        *out_free = total;
        *arrived = 0u; /* every block has arrived */
    }
    if constexpr(PUBLISH)
    {
        const uint32_t n = static_cast<uint32_t>(counts[0]);
        for(uint32_t i = threadIdx.x; i < n; i += kCountThreads)
            out[i] = done[i];
        __syncthreads();
        if(threadIdx.x == 0u)
        {
            *out_len = n;
            *out_remaining = counts[1];
            counts[0] = 0ull;
            counts[1] = 0ull;
        }
    }
}

/* Per-request form: one warp, one slot. */
template<class Ids>
__global__ void mmc_serve_one_kernel(mmc_device_handle h, mmc_serve_slot* slots, mmc_serve_slot* mirror,
                                     void** chunks, uint32_t slot, uint32_t max_chunks, uint32_t step)
{
    if(slots[slot].state != MMC_SERVE_LIVE)
        return;
    grow_request<Ids>(h, slots[slot], chunks + static_cast<uint64_t>(slot) * max_chunks, max_chunks, step);
    __syncwarp();
    if(threadIdx.x == 0u)
        mirror[slot] = slots[slot];
}

namespace
{
    void release(mmc_server* s)
    {
        if(s == nullptr)
            return;
        if(s->exec)
            cudaGraphExecDestroy(s->exec);
        if(s->graph)
            cudaGraphDestroy(s->graph);
        if(s->stream)
            cudaStreamDestroy(s->stream);
        cudaFree(s->d_slots);
        cudaFree(s->d_chunks);
        cudaFreeHost(s->h_queue);
        cudaFreeHost(s->h_queue_len);
        cudaFreeHost(s->h_slots);
        cudaFreeHost(s->h_free);
        if(s->d_count_partials)
            cudaFree(s->d_count_partials);
        if(s->d_count_arrived)
            cudaFree(s->d_count_arrived);
        for(auto& p : s->pipe)
        {
            if(p.exec)
                cudaGraphExecDestroy(p.exec);
            if(p.graph)
                cudaGraphDestroy(p.graph);
            if(p.finished)
                cudaEventDestroy(p.finished);
            cudaFreeHost(p.h_queue);
            cudaFreeHost(p.h_queue_len);
            cudaFreeHost(p.h_done);
            cudaFreeHost(p.h_done_len);
            cudaFreeHost(p.h_remaining);
            cudaFreeHost(p.h_free);
            cudaFree(p.d_done);
            cudaFree(p.d_counts);
        }
        delete s;
    }

    /* The longest request a slot can hold: its chunk row's elements. */
    uint32_t max_request_len(const mmc_server* s)
    {
        const uint64_t n = static_cast<uint64_t>(s->max_chunks) * kElemsPerChunk;
        return n > 0xFFFFFFFFull ? 0xFFFFFFFFu : static_cast<uint32_t>(n);
    }

    /* An admission longer than a slot's chunks hold would index past its row
     * of the chunk table: refused before a tick is launched. */
    mmc_status check_admission_lengths(const mmc_server* s, const mmc_serve_cmd* q, uint32_t n)
    {
        const uint32_t max_len = max_request_len(s);
        for(uint32_t i = 0; i < n; ++i)
            if(q[i].kind == 1u && q[i].final_len > max_len)
                return fail(MMC_ERR_ARG, "command " + std::to_string(i) + " admits " + std::to_string(q[i].final_len)
                                             + " elements; a slot's " + std::to_string(s->max_chunks)
                                             + " chunks hold " + std::to_string(max_len));
        return MMC_OK;
    }

    /* The tick's stream work: queue upload, apply, grow (batched) or not,
     * free-slot count, slot table and count download. */
    mmc_status enqueue_tick(mmc_server* s, bool batched)
    {
        cudaStream_t st = s->stream;
        mmc_serve_apply<<<8, 128, 0, st>>>(s->d_slots, s->m_slots, s->m_queue, s->m_queue_len, s->queue_cap, s->slots,
                                           max_request_len(s), &s->handle.state->error_flags);
        if(batched)
        {
            const uint32_t blocks = (s->slots + 7u) / 8u;
            MMC_DISPATCH_IDS_SIZED(s->handle, kChunkBytes, mmc_serve_tick_kernel<Ids><<<blocks, 256, 0, st>>>(
                                            s->handle, s->d_slots, s->m_slots, s->d_chunks, s->slots, s->max_chunks,
                                            s->step, nullptr, nullptr));
        }
        if(kChunkBytes < s->handle.pagesize)
            mmc_serve_count<false><<<s->count_blocks, kCountThreads, 0, st>>>(
                s->handle, kChunkBytes, s->d_count_partials, s->d_count_arrived, s->m_free, nullptr, nullptr, nullptr,
                nullptr, nullptr);
        else
        {
            mmc_status r = mmc_available_slots_async(s->heap, kChunkBytes, st, s->m_free);
            if(r != MMC_OK)
                return r;
        }
        return cuda_check(cudaGetLastError(), "serve tick");
    }
    /* A pipelined tick on buffer b: apply its queue, grow, count the free
     * chunks into its mapped count, publish its completions. */
    mmc_status enqueue_pipelined_tick(mmc_server* s, int b)
    {
        cudaStream_t st = s->stream;
        mmc_server::Pipe& p = s->pipe[b];
        mmc_serve_apply<<<8, 128, 0, st>>>(s->d_slots, s->m_slots, p.m_queue, p.m_queue_len, s->queue_cap, s->slots,
                                           max_request_len(s), &s->handle.state->error_flags);
        const uint32_t blocks = (s->slots + 7u) / 8u;
        MMC_DISPATCH_IDS_SIZED(s->handle, kChunkBytes, mmc_serve_tick_kernel<Ids><<<blocks, 256, 0, st>>>(
                                        s->handle, s->d_slots, s->m_slots, s->d_chunks, s->slots, s->max_chunks,
                                        s->step, p.d_done, p.d_counts));
        if(kChunkBytes < s->handle.pagesize)
            mmc_serve_count<true><<<s->count_blocks, kCountThreads, 0, st>>>(
                s->handle, kChunkBytes, s->d_count_partials, s->d_count_arrived, p.m_free, p.d_done, p.d_counts,
                p.m_done, p.m_done_len, p.m_remaining);
        else
        {
            mmc_status r = mmc_available_slots_async(s->heap, kChunkBytes, st, p.m_free);
            if(r != MMC_OK)
                return r;
            mmc_serve_publish<<<1, 256, 0, st>>>(p.d_done, p.d_counts, p.m_done, p.m_done_len, p.m_remaining);
        }
        return cuda_check(cudaGetLastError(), "pipelined serve tick");
    }

    /* cudaHostAlloc(mapped) + its device address */
    template<class T>
    mmc_status mapped(T** host, T** dev, size_t bytes, const char* what)
    {
        mmc_status st = cuda_check(cudaHostAlloc(reinterpret_cast<void**>(host), bytes, cudaHostAllocMapped), what);
        if(st == MMC_OK)
            st = cuda_check(cudaHostGetDevicePointer(reinterpret_cast<void**>(dev), *host, 0), what);
        if(st == MMC_OK)
            std::memset(*host, 0, bytes);
        return st;
    }
} // namespace

extern "C" {

mmc_status mmc_serve_create(mmc_heap* heap, uint32_t slots, uint32_t max_chunks, uint32_t step, uint32_t queue_cap,
                            mmc_server** out)
{
    if(heap == nullptr || out == nullptr || slots == 0u || max_chunks == 0u || step == 0u || queue_cap == 0u)
        return fail(MMC_ERR_ARG, "bad server parameters");
    *out = nullptr;
    mmc_server* s = new(std::nothrow) mmc_server();
    if(s == nullptr)
        return fail(MMC_ERR_OOM, "host allocation failed");
    s->heap = heap;
    mmc_heap_device_handle(heap, &s->handle);
    cudaGetDevice(&s->device);
    s->slots = slots;
    s->max_chunks = max_chunks;
    s->step = step;
    s->queue_cap = queue_cap;
    mmc_status st = cuda_check(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "server stream");
    if(st == MMC_OK)
        st = cuda_check(cudaMalloc(&s->d_slots, sizeof(mmc_serve_slot) * slots), "slots");
    if(st == MMC_OK)
        st = cuda_check(cudaMalloc(&s->d_chunks, sizeof(void*) * static_cast<size_t>(slots) * max_chunks), "chunks");
    if(st == MMC_OK)
        st = cuda_check(cudaHostAlloc(&s->h_queue, sizeof(mmc_serve_cmd) * queue_cap, cudaHostAllocMapped),
                        "pinned queue");
    if(st == MMC_OK)
        st = cuda_check(cudaHostAlloc(&s->h_queue_len, sizeof(uint32_t), cudaHostAllocMapped), "pinned queue length");
    if(st == MMC_OK)
        st = cuda_check(cudaHostAlloc(&s->h_slots, sizeof(mmc_serve_slot) * slots, cudaHostAllocMapped),
                        "pinned slots");
    if(st == MMC_OK)
        st = cuda_check(cudaHostAlloc(&s->h_free, sizeof(unsigned), cudaHostAllocMapped), "pinned free count");
    if(st == MMC_OK)
        st = cuda_check(cudaHostGetDevicePointer(reinterpret_cast<void**>(const_cast<mmc_serve_cmd**>(&s->m_queue)),
                                                 s->h_queue, 0),
                        "mapped queue");
    if(st == MMC_OK)
        st = cuda_check(cudaHostGetDevicePointer(reinterpret_cast<void**>(const_cast<uint32_t**>(&s->m_queue_len)),
                                                 s->h_queue_len, 0),
                        "mapped queue length");
    if(st == MMC_OK)
        st = cuda_check(cudaHostGetDevicePointer(reinterpret_cast<void**>(&s->m_slots), s->h_slots, 0),
                        "mapped slots");
    if(st == MMC_OK)
        st = cuda_check(cudaHostGetDevicePointer(reinterpret_cast<void**>(&s->m_free), s->h_free, 0),
                        "mapped free count");
    s->count_blocks = scan_grid(s->device);
    if(st == MMC_OK)
        st = cuda_check(cudaMalloc(&s->d_count_partials, sizeof(uint32_t) * s->count_blocks), "count partials");
    if(st == MMC_OK)
        st = cuda_check(cudaMalloc(&s->d_count_arrived, sizeof(uint32_t)), "count arrivals");
    if(st == MMC_OK)
        st = cuda_check(cudaMemset(s->d_count_arrived, 0, sizeof(uint32_t)), "zero count arrivals");
    if(st == MMC_OK)
        st = cuda_check(cudaMemset(s->d_slots, 0, sizeof(mmc_serve_slot) * slots), "zero slots");
    if(st == MMC_OK)
        st = cuda_check(cudaMemset(s->d_chunks, 0, sizeof(void*) * static_cast<size_t>(slots) * max_chunks),
                        "zero chunks");
    if(st != MMC_OK)
    {
        release(s);
        return st;
    }
    *s->h_queue_len = 0u;
    *s->h_free = 0u;
    std::memset(s->h_slots, 0, sizeof(mmc_serve_slot) * slots);
    /* capture the batched tick once */
    st = cuda_check(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    if(st == MMC_OK)
    {
        mmc_status e = enqueue_tick(s, true);
        st = cuda_check(cudaStreamEndCapture(s->stream, &s->graph), "end capture");
        if(st == MMC_OK)
            st = e;
    }
    if(st == MMC_OK)
        st = cuda_check(cudaGraphInstantiate(&s->exec, s->graph, 0), "instantiate tick graph");
    for(int b = 0; b < 2 && st == MMC_OK; ++b)
    {
        mmc_server::Pipe& p = s->pipe[b];
        mmc_serve_cmd* mq = nullptr;
        uint32_t* mql = nullptr;
        st = mapped(&p.h_queue, &mq, sizeof(mmc_serve_cmd) * queue_cap, "pipelined queue");
        p.m_queue = mq;
        if(st == MMC_OK)
            st = mapped(&p.h_queue_len, &mql, sizeof(uint32_t), "pipelined queue length");
        p.m_queue_len = mql;
        if(st == MMC_OK)
            st = mapped(&p.h_done, &p.m_done, sizeof(mmc_serve_done) * slots, "completion list");
        if(st == MMC_OK)
            st = mapped(&p.h_done_len, &p.m_done_len, sizeof(uint32_t), "completion count");
        if(st == MMC_OK)
            st = mapped(&p.h_remaining, &p.m_remaining, sizeof(unsigned long long), "chunks still to take");
        if(st == MMC_OK)
            st = mapped(&p.h_free, &p.m_free, sizeof(unsigned), "pipelined free count");
        if(st == MMC_OK)
            st = cuda_check(cudaMalloc(&p.d_done, sizeof(mmc_serve_done) * slots), "device completion list");
        if(st == MMC_OK)
            st = cuda_check(cudaMalloc(&p.d_counts, 2 * sizeof(unsigned long long)), "device completion counts");
        if(st == MMC_OK)
            st = cuda_check(cudaMemset(p.d_counts, 0, 2 * sizeof(unsigned long long)), "zero completion counts");
        if(st == MMC_OK)
            st = cuda_check(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        if(st == MMC_OK)
        {
            mmc_status e = enqueue_pipelined_tick(s, b);
            st = cuda_check(cudaStreamEndCapture(s->stream, &p.graph), "end capture");
            if(st == MMC_OK)
                st = e;
        }
        if(st == MMC_OK)
            st = cuda_check(cudaGraphInstantiate(&p.exec, p.graph, 0), "instantiate pipelined tick graph");
        if(st == MMC_OK)
            st = cuda_check(cudaEventCreateWithFlags(&p.finished, cudaEventDisableTiming), "tick event");
    }
    if(st != MMC_OK)
    {
        release(s);
        return st;
    }
    *out = s;
    return MMC_OK;
}

mmc_status mmc_serve_pipeline(mmc_server* s, int buffer, mmc_serve_cmd** queue, uint32_t** queue_len,
                              mmc_serve_done** done, uint32_t** done_len, unsigned long long** remaining,
                              unsigned** free_chunks)
{
    if(s == nullptr || buffer < 0 || buffer > 1)
        return fail(MMC_ERR_ARG, "server is null or buffer not 0 or 1");
    mmc_server::Pipe& p = s->pipe[buffer];
    if(queue)
        *queue = p.h_queue;
    if(queue_len)
        *queue_len = p.h_queue_len;
    if(done)
        *done = p.h_done;
    if(done_len)
        *done_len = p.h_done_len;
    if(remaining)
        *remaining = p.h_remaining;
    if(free_chunks)
        *free_chunks = p.h_free;
    return MMC_OK;
}

mmc_status mmc_serve_check_queue(const mmc_serve_cmd* queue, uint32_t queue_len, uint32_t queue_cap, uint32_t slots)
{
    if(queue_len > queue_cap)
        return fail(MMC_ERR_ARG, "queue length " + std::to_string(queue_len) + " exceeds the queue's capacity of "
                                     + std::to_string(queue_cap) + " commands");
    if(queue_len != 0u && queue == nullptr)
        return fail(MMC_ERR_ARG, "queue is null");
    for(uint32_t i = 0; i < queue_len; ++i)
    {
        if(queue[i].kind != 1u && queue[i].kind != 2u)
            return fail(MMC_ERR_ARG, "command " + std::to_string(i) + " has unknown kind "
                                         + std::to_string(queue[i].kind));
        if(queue[i].slot >= slots)
            return fail(MMC_ERR_ARG, "command " + std::to_string(i) + " names slot " + std::to_string(queue[i].slot)
                                         + " of a table of " + std::to_string(slots));
    }
    return MMC_OK;
}

mmc_status mmc_serve_launch(mmc_server* s, int buffer)
{
    mmc::host::NvtxRange nvtx_range("mmc_serve_launch");
    if(s == nullptr || buffer < 0 || buffer > 1)
        return fail(MMC_ERR_ARG, "server is null or buffer not 0 or 1");
    /* the tick on this buffer reads the queue the host has just written: check it first */
    mmc_status q = mmc_serve_check_queue(s->pipe[buffer].h_queue, *s->pipe[buffer].h_queue_len, s->queue_cap,
                                         s->slots);
    if(q == MMC_OK)
        q = check_admission_lengths(s, s->pipe[buffer].h_queue, *s->pipe[buffer].h_queue_len);
    if(q != MMC_OK)
        return q;
    mmc_status st = cuda_check(cudaGraphLaunch(s->pipe[buffer].exec, s->stream), "pipelined tick launch");
    if(st == MMC_OK)
        st = cuda_check(cudaEventRecord(s->pipe[buffer].finished, s->stream), "record tick event");
    return st;
}

mmc_status mmc_serve_wait_buffer(mmc_server* s, int buffer)
{
    if(s == nullptr || buffer < 0 || buffer > 1)
        return fail(MMC_ERR_ARG, "server is null or buffer not 0 or 1");
    return cuda_check(cudaEventSynchronize(s->pipe[buffer].finished), "wait for tick");
}

mmc_status mmc_serve_wait(mmc_server* s)
{
    if(s == nullptr)
        return fail(MMC_ERR_ARG, "server is null");
    return cuda_check(cudaStreamSynchronize(s->stream), "wait for ticks");
}

mmc_status mmc_serve_queue(mmc_server* s, mmc_serve_cmd** queue, uint32_t** queue_len, mmc_serve_slot** slots,
                           unsigned** free_chunks)
{
    if(s == nullptr)
        return fail(MMC_ERR_ARG, "server is null");
    if(queue)
        *queue = s->h_queue;
    if(queue_len)
        *queue_len = s->h_queue_len;
    if(slots)
        *slots = s->h_slots;
    if(free_chunks)
        *free_chunks = s->h_free;
    return MMC_OK;
}

mmc_status mmc_serve_tick(mmc_server* s, int batched)
{
    mmc::host::NvtxRange nvtx_range("mmc_serve_tick");
    if(s == nullptr)
        return fail(MMC_ERR_ARG, "server is null");
    mmc_status st = mmc_serve_check_queue(s->h_queue, *s->h_queue_len, s->queue_cap, s->slots);
    if(st == MMC_OK)
        st = check_admission_lengths(s, s->h_queue, *s->h_queue_len);
    if(st != MMC_OK)
        return st;
    if(batched)
        st = cuda_check(cudaGraphLaunch(s->exec, s->stream), "tick graph launch");
    else
    {
        /* one grow launch per live request (from the host copy of the table),
         * around the same apply / count / download steps */
        cudaStream_t stream = s->stream;
        /* which slots are live after this tick's admissions and releases, from
         * the host's table and queue, before the apply kernel has run */
        std::vector<uint8_t> live(s->slots, 0u);
        for(uint32_t w = 0; w < s->slots; ++w)
            live[w] = s->h_slots[w].state == MMC_SERVE_LIVE;
        for(uint32_t i = 0; i < *s->h_queue_len; ++i)
            live[s->h_queue[i].slot] = s->h_queue[i].kind == 1u;
        mmc_serve_apply<<<8, 128, 0, stream>>>(s->d_slots, s->m_slots, s->m_queue, s->m_queue_len, s->queue_cap,
                                               s->slots, max_request_len(s), &s->handle.state->error_flags);
        for(uint32_t w = 0; w < s->slots; ++w)
            if(live[w])
                MMC_DISPATCH_IDS_SIZED(s->handle, kChunkBytes, mmc_serve_one_kernel<Ids><<<1, 32, 0, stream>>>(
                                                s->handle, s->d_slots, s->m_slots, s->d_chunks, w, s->max_chunks,
                                                s->step));
        st = mmc_available_slots_async(s->heap, kChunkBytes, stream, s->m_free);
        if(st == MMC_OK)
            st = cuda_check(cudaGetLastError(), "per-request tick");
    }
    if(st == MMC_OK)
        st = cuda_check(cudaStreamSynchronize(s->stream), "tick");
    return st;
}

mmc_status mmc_serve_destroy(mmc_server* s)
{
    if(s == nullptr)
        return MMC_OK;
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->stream);
    release(s);
    return MMC_OK;
}

} /* extern "C" */

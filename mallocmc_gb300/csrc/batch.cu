/* batch.cu — many independent allocation jobs on one heap, in one launch.
 *
 * A job is `threads` threads, each running `cycles` (drawn per thread in
 * [min_cycles, max_cycles]) of {malloc(size), write a u64 pattern, verify it,
 * free}; sizes are geometric with mean `mean_size` bytes, capped at `max_size`
 * and padded to 16 (all draws seeded per job, thread and cycle, so every form
 * of the launch performs the same allocations).
 *
 * Two forms of the same work:
 *   plain       one kernel launch per job (grid = ceil(threads / 256))
 *   persistent  one launch of a fixed grid whose lanes take job threads
 *               from a device counter until the batch is done: a lane whose
 *               thread has run its last cycle takes the next one at once, so
 *               no warp idles while its slowest lane finishes (cycle counts
 *               differ by up to 16x within a warp). The counter reset and the
 *               launch are captured once into a CUDA graph and replayed per run.
 * Per-job counters {pairs, nulls, pattern errors, checksum} make the forms
 * comparable job by job.
 */
#include "mmc_internal.h"

#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

using namespace mmc::host;
namespace dv = mmc::dev;

struct mmc_batch
{
    mmc_heap* heap;
    mmc_device_handle handle;
    int device;
    uint32_t njobs;
    uint32_t total_items;
    uint32_t blocks;
    uint32_t threads_per_block;
    std::vector<mmc_job> host_jobs;
    mmc_job* jobs;              /* device copy, item_begin filled */
    uint32_t* item_job;         /* job of each 256-thread work item (total_items entries) */
    unsigned long long* counter; /* job-thread counter of the persistent form */
    bool shared_rows;            /* per-block pair/checksum columns fit shared memory and u32 */
    uint32_t max_request;        /* the largest max_size of the jobs (a request's bytes before padding) */
    unsigned long long* stats;  /* njobs x 4 */
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    cudaStream_t capture_stream;
};

namespace
{
    constexpr uint32_t kItemThreads = 256;
    /* per-block pair and checksum columns in shared memory up to 32 KiB
     * (2730 jobs); larger batches flush to the global table directly */
    constexpr size_t kSharedRowsMax = 32u << 10;

    __host__ __device__ __forceinline__ uint64_t mix64(uint64_t seed, uint64_t a, uint64_t b)
    {
        uint64_t z = seed + a * 0x9E3779B97F4A7C15ull + b * 0xD1B54A32D192ED03ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }

    /* Size of cycle c of job thread jt: geometric on {1, 2, ...} with the job's
     * mean (inverse-CDF draw), capped, padded to 16. */
    __device__ __forceinline__ float log_q(const mmc_job& j)
    {
        return logf(1.0f - 1.0f / static_cast<float>(j.mean_size));
    }

    /* logq = log_q(j), which a caller running many cycles of one job computes once */
    __device__ __forceinline__ uint32_t draw_size(const mmc_job& j, uint64_t m, float logq)
    {
        const float u = (static_cast<float>(m >> 40) + 0.5f) * (1.0f / 16777216.0f); /* (0, 1) */
        float x = 1.0f + floorf(logf(u) / logq);
        if(!(x < static_cast<float>(j.max_size)))
            x = static_cast<float>(j.max_size);
        const uint32_t s = static_cast<uint32_t>(x);
        return (s + 15u) & ~15u;
    }

    template<class Ids>
    __device__ __forceinline__ void run_job_thread(const mmc_device_handle& h, const mmc_job& j, uint32_t jt,
                                                   unsigned long long& pairs, unsigned long long& nulls,
                                                   unsigned long long& bad, unsigned long long& csum)
    {
        const uint32_t span = j.max_cycles - j.min_cycles + 1u;
        const uint32_t cycles = j.min_cycles + static_cast<uint32_t>(mix64(j.seed, jt, 0xC1C1Eull) >> 32) % span;
        const float logq = log_q(j);
        for(uint32_t c = 0; c < cycles; ++c)
        {
            const uint64_t m = mix64(j.seed, jt, c);
            const uint32_t bytes = draw_size(j, m, logq);
            char* ptr = static_cast<char*>(dv::malloc<Ids>(h, bytes));
            if(ptr == nullptr)
            {
                ++nulls;
                continue;
            }
            ulonglong2* q = reinterpret_cast<ulonglong2*>(ptr);
            const uint32_t n16 = bytes / 16u;
            for(uint32_t i = 0; i < n16; ++i)
                q[i] = make_ulonglong2(m + 2u * i, m + 2u * i + 1u);
            for(uint32_t i = 0; i < n16; ++i)
            {
                const ulonglong2 v = q[i];
                bad += (v.x != m + 2u * i) + (v.y != m + 2u * i + 1u);
                csum += v.x ^ v.y;
            }
            dv::free<Ids>(h, ptr);
            ++pairs;
        }
    }

    __device__ __forceinline__ void flush_stats(unsigned long long* s, unsigned long long pairs,
                                                unsigned long long nulls, unsigned long long bad,
                                                unsigned long long csum)
    {
        /* every lane of the warp calls this (the kernels never exit lanes early) */
        __syncwarp();
        for(int off = 16; off > 0; off >>= 1)
        {
            pairs += __shfl_down_sync(0xFFFFFFFFu, pairs, off);
            nulls += __shfl_down_sync(0xFFFFFFFFu, nulls, off);
            bad += __shfl_down_sync(0xFFFFFFFFu, bad, off);
            csum ^= __shfl_down_sync(0xFFFFFFFFu, csum, off);
        }
        if((threadIdx.x & 31u) == 0u)
        {
            if(pairs)
                atomicAdd(&s[0], pairs);
            if(nulls)
                atomicAdd(&s[1], nulls);
            if(bad)
                atomicAdd(&s[2], bad);
            if(csum)
                atomicXor(&s[3], csum);
        }
    }
} // namespace

/* Plain form: one launch per job. */
template<class Ids>
__global__ void __launch_bounds__(256) mmc_job_kernel(mmc_device_handle h, const mmc_job* jobs, uint32_t job,
                                                      unsigned long long* stats)
{
    const mmc_job j = jobs[job];
    const uint32_t jt = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long pairs = 0, nulls = 0, bad = 0, csum = 0;
    if(jt < j.threads)
        run_job_thread<Ids>(h, j, jt, pairs, nulls, bad, csum);
    flush_stats(stats + 4ull * job, pairs, nulls, bad, csum);
}

/* Persistent form. Job threads are numbered in work-item space: job i owns
 * slots [256 * item_begin_i, 256 * item_begin_i + threads_i); the slots up to
 * the next job's first item are padding and are skipped. Every lane runs one
 * job thread at a time, one cycle per pass of the loop; lanes that need a
 * thread take consecutive slots with one atomicAdd per warp, and a table of
 * each work item's job (built with the batch) names the slot's job in one
 * load. A lane's counters
 * are flushed to its job's row when it leaves a thread. With SHARED_ROWS the
 * pairs and the checksum (the words every thread adds to) go to the block's
 * copy of those two columns in shared memory (12 B per job), which the block
 * adds to the global table once at its end; without, and for the rare null and
 * pattern-error counts, straight to the global table. (One thread's flush to
 * L2 is two atomics, more than its share of the allocations' atomics.) Four
 * resident blocks per SM (64 registers, a few spilled) against three at the
 * unbounded 80: 7 % faster on the tuned geometry, 4.5 % on the defaults. */
template<bool SHARED_ROWS, class Ids>
__global__ void __launch_bounds__(256, 4) mmc_batch_kernel(mmc_device_handle h, const mmc_job* jobs,
                                                        const uint32_t* item_job, uint32_t njobs,
                                                        unsigned long long total_slots, unsigned long long* counter,
                                                        unsigned long long* stats)
{
    extern __shared__ unsigned long long s_csum[]; /* njobs checksums, then njobs u32 pair counts */
    uint32_t* s_pairs = reinterpret_cast<uint32_t*>(s_csum + njobs);
    if constexpr(SHARED_ROWS)
    {
        for(uint32_t i = threadIdx.x; i < njobs; i += blockDim.x)
        {
            s_csum[i] = 0ull;
            s_pairs[i] = 0u;
        }
        __syncthreads();
    }
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lanes_below = (1u << lane) - 1u;
    uint32_t job = 0, jt = 0, cycles = 0, c = 0;
    uint64_t seed = 0;
    float logq = 0.0f;
    mmc_job j{};
    bool done = false;
    /* 32-bit per-thread counts (a job thread runs at most max_cycles): at
     * the kernel's 64-register bound, registers the loop need not spill */
    uint32_t pairs = 0, nulls = 0, bad = 0;
    unsigned long long csum = 0;
    for(;;)
    {
        bool need = !done && c == cycles;
        unsigned needm = __ballot_sync(0xFFFFFFFFu, need);
        while(needm != 0u)
        {
            const int leader = __ffs(static_cast<int>(needm)) - 1;
            unsigned long long base = 0;
            if(static_cast<int>(lane) == leader)
                base = atomicAdd(counter, static_cast<unsigned long long>(__popc(needm)));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            if(need)
            {
                if(cycles != 0u)
                {
                    unsigned long long* s = stats + 4ull * job;
                    if constexpr(SHARED_ROWS)
                    {
                        atomicAdd(&s_pairs[job], pairs);
                        atomicXor(&s_csum[job], csum);
                    }
                    else
                    {
                        atomicAdd(&s[0], static_cast<unsigned long long>(pairs));
                        atomicXor(&s[3], csum);
                    }
                    if(nulls)
                        atomicAdd(&s[1], static_cast<unsigned long long>(nulls));
                    if(bad)
                        atomicAdd(&s[2], static_cast<unsigned long long>(bad));
                    pairs = nulls = bad = csum = 0;
                    cycles = c = 0;
                }
                const unsigned long long slot = base + static_cast<unsigned>(__popc(needm & lanes_below));
                if(slot >= total_slots)
                {
                    done = true;
                    need = false;
                }
                else
                {
                    job = item_job[static_cast<uint32_t>(slot / kItemThreads)];
                    j = jobs[job];
                    jt = static_cast<uint32_t>(slot - static_cast<unsigned long long>(j.item_begin) * kItemThreads);
                    if(jt < j.threads)
                    {
                        const uint32_t span = j.max_cycles - j.min_cycles + 1u;
                        cycles = j.min_cycles + static_cast<uint32_t>(mix64(j.seed, jt, 0xC1C1Eull) >> 32) % span;
                        seed = j.seed;
                        logq = log_q(j);
                        need = cycles == 0u; /* a thread with no cycles is done at once */
                    }
                }
            }
            needm = __ballot_sync(0xFFFFFFFFu, need);
        }
        if(__all_sync(0xFFFFFFFFu, done))
            break;
        if(!done)
        {
            const uint64_t m = mix64(seed, jt, c);
            const uint32_t bytes = draw_size(j, m, logq);
            char* ptr = static_cast<char*>(dv::malloc<Ids>(h, bytes));
            if(ptr == nullptr)
                ++nulls;
            else
            {
                ulonglong2* q = reinterpret_cast<ulonglong2*>(ptr);
                const uint32_t n16 = bytes / 16u;
                for(uint32_t i = 0; i < n16; ++i)
                    q[i] = make_ulonglong2(m + 2u * i, m + 2u * i + 1u);
                for(uint32_t i = 0; i < n16; ++i)
                {
                    const ulonglong2 v = q[i];
                    bad += (v.x != m + 2u * i) + (v.y != m + 2u * i + 1u);
                    csum += v.x ^ v.y;
                }
                dv::free<Ids>(h, ptr);
                ++pairs;
            }
            ++c;
        }
    }
    if constexpr(SHARED_ROWS)
    {
        __syncthreads();
        for(uint32_t i = threadIdx.x; i < njobs; i += blockDim.x)
        {
            if(s_pairs[i] != 0u)
                atomicAdd(&stats[4ull * i], static_cast<unsigned long long>(s_pairs[i]));
            if(s_csum[i] != 0ull)
                atomicXor(&stats[4ull * i + 3u], s_csum[i]);
        }
    }
}

namespace
{
    void release(mmc_batch* b)
    {
        if(b == nullptr)
            return;
        if(b->exec)
            cudaGraphExecDestroy(b->exec);
        if(b->graph)
            cudaGraphDestroy(b->graph);
        if(b->capture_stream)
            cudaStreamDestroy(b->capture_stream);
        if(b->jobs)
            cudaFree(b->jobs);
        if(b->counter)
            cudaFree(b->counter);
        if(b->stats)
            cudaFree(b->stats);
        if(b->item_job)
            cudaFree(b->item_job);
        delete b;
    }

    void launch_persistent(mmc_batch* b, cudaStream_t s)
    {
        cudaMemsetAsync(b->counter, 0, sizeof(unsigned long long), s);
        const unsigned long long slots = static_cast<unsigned long long>(b->total_items) * kItemThreads;
        const size_t rows_bytes = (sizeof(unsigned long long) + sizeof(uint32_t)) * b->njobs;
        MMC_DISPATCH_IDS_SIZED(b->handle, b->max_request, if(b->shared_rows) mmc_batch_kernel<true, Ids>
                                        <<<b->blocks, kItemThreads, rows_bytes, s>>>(b->handle, b->jobs, b->item_job,
                                                                                     b->njobs, slots, b->counter,
                                                                                     b->stats);
                         else mmc_batch_kernel<false, Ids><<<b->blocks, kItemThreads, 0, s>>>(
                             b->handle, b->jobs, b->item_job, b->njobs, slots, b->counter, b->stats));
    }
} // namespace

extern "C" {

mmc_status mmc_batch_create(mmc_heap* heap, const mmc_job* jobs, uint32_t njobs, uint32_t persistent_blocks,
                            int use_graph, void* stream, mmc_batch** out)
{
    if(heap == nullptr || jobs == nullptr || out == nullptr || njobs == 0u)
        return fail(MMC_ERR_ARG, "null argument or empty batch");
    *out = nullptr;
    mmc_batch* b = new(std::nothrow) mmc_batch();
    if(b == nullptr)
        return fail(MMC_ERR_OOM, "host allocation failed");
    mmc_heap_device_handle(heap, &b->handle);
    b->heap = heap;
    cudaGetDevice(&b->device);
    b->njobs = njobs;
    b->threads_per_block = kItemThreads;
    b->host_jobs.assign(jobs, jobs + njobs);
    uint64_t items = 0;
    for(auto& j : b->host_jobs)
    {
        if(j.threads == 0u || j.mean_size == 0u || j.max_size == 0u || j.min_cycles > j.max_cycles)
        {
            release(b);
            return fail(MMC_ERR_ARG, "bad job descriptor");
        }
        j.item_begin = static_cast<uint32_t>(items);
        items += (j.threads + kItemThreads - 1u) / kItemThreads;
        b->max_request = std::max(b->max_request, j.max_size);
    }
    if(items > 0xFFFFFFF0ull)
    {
        release(b);
        return fail(MMC_ERR_ARG, "batch too large");
    }
    b->total_items = static_cast<uint32_t>(items);
    b->shared_rows = (sizeof(unsigned long long) + sizeof(uint32_t)) * njobs <= kSharedRowsMax;
    for(const auto& j : b->host_jobs)
        if(static_cast<uint64_t>(j.threads) * j.max_cycles > 0xFFFFFFFFull)
            b->shared_rows = false; /* a block's pair count of the job could pass 32 bits */
    b->blocks = persistent_blocks ? persistent_blocks : scan_grid(b->device) * 2u;
    cudaStream_t s = as_stream(stream);
    std::vector<uint32_t> item_job(b->total_items);
    for(uint32_t i = 0; i < njobs; ++i)
    {
        const uint32_t end = i + 1u < njobs ? b->host_jobs[i + 1u].item_begin : b->total_items;
        for(uint32_t it = b->host_jobs[i].item_begin; it < end; ++it)
            item_job[it] = i;
    }
    mmc_status st = cuda_check(cudaMalloc(&b->jobs, sizeof(mmc_job) * njobs), "cudaMalloc jobs");
    if(st == MMC_OK)
        st = cuda_check(cudaMalloc(&b->item_job, sizeof(uint32_t) * (b->total_items > 0u ? b->total_items : 1u)),
                        "cudaMalloc item table");
    if(st == MMC_OK && b->total_items > 0u)
        st = cuda_check(cudaMemcpyAsync(b->item_job, item_job.data(), sizeof(uint32_t) * b->total_items,
                                        cudaMemcpyHostToDevice, s),
                        "copy item table");
    if(st == MMC_OK)
        st = cuda_check(cudaMalloc(&b->counter, sizeof(unsigned long long)), "cudaMalloc counter");
    if(st == MMC_OK)
        st = cuda_check(cudaMalloc(&b->stats, sizeof(unsigned long long) * 4ull * njobs), "cudaMalloc stats");
    if(st == MMC_OK)
        st = cuda_check(cudaMemcpyAsync(b->jobs, b->host_jobs.data(), sizeof(mmc_job) * njobs, cudaMemcpyHostToDevice, s),
                        "copy jobs");
    if(st == MMC_OK)
        st = cuda_check(cudaMemsetAsync(b->stats, 0, sizeof(unsigned long long) * 4ull * njobs, s), "zero stats");
    if(st == MMC_OK)
        st = cuda_check(cudaStreamSynchronize(s), "wait for batch upload");
    if(st == MMC_OK && use_graph)
    {
        st = cuda_check(cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking), "capture stream");
        if(st == MMC_OK)
            st = cuda_check(cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal),
                            "begin capture");
        if(st == MMC_OK)
        {
            launch_persistent(b, b->capture_stream);
            st = cuda_check(cudaStreamEndCapture(b->capture_stream, &b->graph), "end capture");
        }
        if(st == MMC_OK)
            st = cuda_check(cudaGraphInstantiate(&b->exec, b->graph, 0), "instantiate graph");
    }
    if(st != MMC_OK)
    {
        release(b);
        return st;
    }
    *out = b;
    return MMC_OK;
}

mmc_status mmc_batch_run(mmc_batch* b, void* stream)
{
    mmc::host::NvtxRange nvtx_range("mmc_batch_run");
    if(b == nullptr)
        return fail(MMC_ERR_ARG, "batch is null");
    cudaStream_t s = as_stream(stream);
    if(b->exec)
        return cuda_check(cudaGraphLaunch(b->exec, s), "graph launch");
    launch_persistent(b, s);
    return cuda_check(cudaGetLastError(), "persistent batch kernel");
}

mmc_status mmc_batch_run_plain(mmc_batch* b, void* stream)
{
    mmc::host::NvtxRange nvtx_range("mmc_batch_run_plain");
    if(b == nullptr)
        return fail(MMC_ERR_ARG, "batch is null");
    cudaStream_t s = as_stream(stream);
    for(uint32_t i = 0; i < b->njobs; ++i)
    {
        const uint32_t grid = (b->host_jobs[i].threads + kItemThreads - 1u) / kItemThreads;
        MMC_DISPATCH_IDS_SIZED(b->handle, b->host_jobs[i].max_size,
                               mmc_job_kernel<Ids><<<grid, kItemThreads, 0, s>>>(b->handle, b->jobs, i, b->stats));
    }
    return cuda_check(cudaGetLastError(), "plain job kernels");
}

mmc_status mmc_batch_stats(mmc_batch* b, void* stream, unsigned long long* out, int clear)
{
    if(b == nullptr || out == nullptr)
        return fail(MMC_ERR_ARG, "null argument");
    cudaStream_t s = as_stream(stream);
    mmc_status st = cuda_check(cudaMemcpyAsync(out, b->stats, sizeof(unsigned long long) * 4ull * b->njobs,
                                               cudaMemcpyDeviceToHost, s),
                               "copy batch stats");
    if(st == MMC_OK && clear)
        st = cuda_check(cudaMemsetAsync(b->stats, 0, sizeof(unsigned long long) * 4ull * b->njobs, s), "clear stats");
    if(st == MMC_OK)
        st = cuda_check(cudaStreamSynchronize(s), "wait for batch stats");
    return st;
}

mmc_status mmc_batch_info(const mmc_batch* b, uint32_t* total_items, uint32_t* blocks, uint64_t* total_threads)
{
    if(b == nullptr)
        return fail(MMC_ERR_ARG, "batch is null");
    if(total_items)
        *total_items = b->total_items;
    if(blocks)
        *blocks = b->blocks;
    if(total_threads)
    {
        uint64_t t = 0;
        for(const auto& j : b->host_jobs)
            t += j.threads;
        *total_threads = t;
    }
    return MMC_OK;
}

mmc_status mmc_batch_destroy(mmc_batch* b)
{
    if(b == nullptr)
        return MMC_OK;
    cudaSetDevice(b->device);
    cudaDeviceSynchronize();
    release(b);
    return MMC_OK;
}

} /* extern "C" */

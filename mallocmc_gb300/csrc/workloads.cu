/* workloads.cu — kernels built on the device API (mallocMC/scatter_device.cuh),
 * exported through the C ABI for verification and benchmarking:
 *   mmc_run_program   one device thread replays an op program with the reference
 *                     CPU backend's thread ids (bit-exact offsets);
 *   mmc_run_stress    every thread: rounds x {malloc, write u64 pattern, verify, free};
 *   mmc_run_verify    the plain verify workload (u32 pattern t ^ seed), and its
 *                     alloc / free halves for inspecting the heap in between.
 * These are what user kernels do with handle.malloc / handle.free
 * (tests/verify_heap.cpp:333-388 in the reference is the pattern).
 */
#include "mmc_internal.h"

#include <algorithm>

using namespace mmc::host;
namespace dv = mmc::dev;

namespace
{
    __host__ __device__ __forceinline__ uint64_t mix64(uint64_t seed, uint64_t a, uint64_t b)
    {
        uint64_t z = seed + a * 0x9E3779B97F4A7C15ull + b * 0xD1B54A32D192ED03ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
} // namespace

/* One thread, SerialIds: the reference's CPU-serial semantics. */
__global__ void mmc_program_kernel(mmc_device_handle h, const uint8_t* kinds, const uint64_t* args, int64_t begin,
                                   int64_t end, int64_t* out)
{
    if(blockIdx.x != 0 || threadIdx.x != 0)
        return;
    for(int64_t i = begin; i < end; ++i)
    {
        const uint8_t k = kinds[i];
        if(k == 'm')
        {
            void* p = dv::malloc<dv::SerialIds>(h, static_cast<size_t>(args[i]));
            out[i] = p ? static_cast<int64_t>(static_cast<char*>(p) - h.pages) : -1;
        }
        else if(k == 'f')
        {
            const int64_t j = static_cast<int64_t>(args[i]);
            if(j >= 0 && j < i && kinds[j] == 'm' && out[j] >= 0)
                dv::free<dv::SerialIds>(h, h.pages + out[j]);
            out[i] = 0;
        }
        else if(k == 'd')
            out[i] = dv::available_slots<dv::SerialIds>(h, static_cast<size_t>(args[i]));
        else
            out[i] = 0;
    }
}

__global__ void mmc_store_result_kernel(const unsigned* src, int64_t* dst) { *dst = static_cast<int64_t>(*src); }

constexpr uint32_t kPatternGroup = 2u; /* blocks whose read-back is in flight together */

/* Write then verify the u64 pattern m + i of `bytes` bytes at every lane's
 * block, cooperatively: the warp walks the blocks of its lanes in turn and
 * moves 512 contiguous bytes per instruction (16 per lane), instead of each
 * lane streaming its own block 16 bytes at a time across 32 cache lines.
 * The read-back issues the first 1 KiB of kPatternGroup blocks before it
 * compares any, so their loads are in flight together. Each lane reads back
 * the 16-byte units it wrote (units lane, lane + 32, ... of every block).
 * Every lane of the warp must call it (blocks of lanes whose ptr is null are
 * skipped). Returns the pattern mismatches found in this lane's share. */
__device__ __forceinline__ uint32_t warp_pattern(char* ptr, uint32_t bytes, uint64_t m, unsigned long long& csum)
{
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t bad = 0;
    const unsigned have = __ballot_sync(0xFFFFFFFFu, ptr != nullptr);
    for(unsigned rest = have; rest != 0u; rest &= rest - 1u)
    {
        const int k = __ffs(static_cast<int>(rest)) - 1;
        ulonglong2* q = reinterpret_cast<ulonglong2*>(__shfl_sync(0xFFFFFFFFu, reinterpret_cast<unsigned long long>(ptr), k));
        const uint32_t n16 = __shfl_sync(0xFFFFFFFFu, bytes, k) / 16u;
        const uint64_t mk = __shfl_sync(0xFFFFFFFFu, m, k);
        for(uint32_t i = lane; i < n16; i += 32u)
            q[i] = make_ulonglong2(mk + 2u * i, mk + 2u * i + 1u);
    }
    __syncwarp();
    for(unsigned rest = have; rest != 0u;)
    {
        const ulonglong2* q[kPatternGroup];
        uint32_t n16[kPatternGroup];
        uint64_t mk[kPatternGroup];
#pragma unroll
        for(uint32_t j = 0; j < kPatternGroup; ++j)
        {
            const bool live = rest != 0u;
            const int k = live ? __ffs(static_cast<int>(rest)) - 1 : 0;
            rest &= rest - 1u;
            q[j] = reinterpret_cast<const ulonglong2*>(
                __shfl_sync(0xFFFFFFFFu, reinterpret_cast<unsigned long long>(ptr), k));
            const uint32_t nk = __shfl_sync(0xFFFFFFFFu, bytes, k) / 16u;
            n16[j] = live ? nk : 0u;
            mk[j] = __shfl_sync(0xFFFFFFFFu, m, k);
        }
        ulonglong2 v[kPatternGroup][2];
#pragma unroll
        for(uint32_t j = 0; j < kPatternGroup; ++j)
        {
#pragma unroll
            for(uint32_t u = 0; u < 2u; ++u)
            {
                const uint32_t i = lane + 32u * u;
                v[j][u] = i < n16[j] ? q[j][i] : make_ulonglong2(0ull, 0ull);
            }
        }
#pragma unroll
        for(uint32_t j = 0; j < kPatternGroup; ++j)
        {
#pragma unroll
            for(uint32_t u = 0; u < 2u; ++u)
            {
                const uint32_t i = lane + 32u * u;
                if(i < n16[j])
                {
                    bad += (v[j][u].x != mk[j] + 2u * i) + (v[j][u].y != mk[j] + 2u * i + 1u);
                    csum += v[j][u].x ^ v[j][u].y;
                }
            }
            /* blocks above 1 KiB: the rest one 512-byte row at a time */
            for(uint32_t i = lane + 64u; i < n16[j]; i += 32u)
            {
                const ulonglong2 w = q[j][i];
                bad += (w.x != mk[j] + 2u * i) + (w.y != mk[j] + 2u * i + 1u);
                csum += w.x ^ w.y;
            }
        }
    }
    __syncwarp();
    return bad;
}

/* Uniform stress: sizes[r * nthreads + t] or drawn from the seed. Launch
 * bounds of four 256-thread CTAs per SM (64 registers): that build measured
 * about 6 % faster on GB300 than the one without the bound. With the warp
 * pattern, each verified block's whole cache lines are dropped from L2
 * (discard_dead_block) before it is freed: the block is dead, and its
 * payload would otherwise be written back to DRAM (6 % faster). */
template<uint32_t PATTERN, class Ids>
__global__ void __launch_bounds__(256, 4) mmc_stress_kernel(mmc_device_handle h, mmc_stress_params p,
                                                         const uint16_t* sizes, unsigned long long* stats)
{
    /* 32-bit thread index and per-thread counts (a thread counts at most
     * `rounds` pairs): at the kernel's 64-register bound every register the
     * loop keeps live is one the allocator need not spill */
    const uint32_t nthreads = gridDim.x * blockDim.x;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nsizes = (p.hi - p.lo) / p.step + 1u;
    uint32_t pairs = 0, nulls = 0, bad = 0;
    unsigned long long csum = 0;
    for(uint32_t r = 0; r < p.rounds; ++r)
    {
        const uint64_t m = mix64(p.seed, t, r);
        const uint32_t bytes = sizes ? sizes[static_cast<uint64_t>(r) * nthreads + t]
                                     : p.lo + (static_cast<uint32_t>(m >> 32) % nsizes) * p.step;
        char* ptr = static_cast<char*>(dv::malloc<Ids>(h, bytes));
        if constexpr(PATTERN == MMC_PATTERN_WARP)
        {
            /* every lane takes part, with or without a block */
            bad += warp_pattern(ptr, bytes, m, csum);
            if(ptr == nullptr)
                ++nulls;
            else
            {
                /* the verified block is dead: its whole lines leave L2 unwritten */
                dv::free<Ids>(h, dv::discard_dead_block(ptr, bytes));
                ++pairs;
            }
            continue;
        }
        if(ptr == nullptr)
        {
            ++nulls;
            continue;
        }
        if constexpr(PATTERN == MMC_PATTERN_THREAD)
        {
            /* 16-byte stores: chunks are 16-byte aligned under Shrink<16> */
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
        }
        dv::free<Ids>(h, ptr);
        ++pairs;
    }
    /* warp-aggregate the counters */
    for(int off = 16; off > 0; off >>= 1)
    {
        pairs += __shfl_down_sync(0xFFFFFFFFu, pairs, off);
        nulls += __shfl_down_sync(0xFFFFFFFFu, nulls, off);
        bad += __shfl_down_sync(0xFFFFFFFFu, bad, off);
        csum ^= __shfl_down_sync(0xFFFFFFFFu, csum, off);
    }
    if((threadIdx.x & 31u) == 0u)
    {
        atomicAdd(&stats[0], static_cast<unsigned long long>(pairs));
        if(nulls)
            atomicAdd(&stats[1], static_cast<unsigned long long>(nulls));
        if(bad)
            atomicAdd(&stats[2], static_cast<unsigned long long>(bad));
        atomicXor(&stats[3], csum);
    }
}

/* The same stress on CUDA's device heap (CreationPolicies::OldMalloc, OldMalloc.hpp:59-68). */
__global__ void __launch_bounds__(256) mmc_stress_oldmalloc_kernel(mmc_stress_params p, const uint16_t* sizes,
                                                                   unsigned long long* stats)
{
    const uint64_t nthreads = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    const uint64_t t = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const uint32_t nsizes = (p.hi - p.lo) / p.step + 1u;
    unsigned long long pairs = 0, nulls = 0, bad = 0, csum = 0;
    for(uint32_t r = 0; r < p.rounds; ++r)
    {
        const uint64_t m = mix64(p.seed, t, r);
        const uint32_t bytes
            = sizes ? sizes[r * nthreads + t] : p.lo + (static_cast<uint32_t>(m >> 32) % nsizes) * p.step;
        char* ptr = static_cast<char*>(::malloc(bytes));
        if(p.write_pattern == MMC_PATTERN_WARP)
        {
            bad += warp_pattern(ptr, bytes, m, csum);
            if(ptr == nullptr)
                ++nulls;
            else
            {
                /* as the GB300 heap's stress does; CUDA's free is given the
                 * same release fence the Scatter free issues itself */
                dv::discard_dead_block(ptr, bytes);
                dv::release_fence();
                ::free(ptr);
                ++pairs;
            }
            continue;
        }
        if(ptr == nullptr)
        {
            ++nulls;
            continue;
        }
        if(p.write_pattern == MMC_PATTERN_THREAD)
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
        }
        dv::release_fence();
        ::free(ptr);
        ++pairs;
    }
    for(int off = 16; off > 0; off >>= 1)
    {
        pairs += __shfl_down_sync(0xFFFFFFFFu, pairs, off);
        nulls += __shfl_down_sync(0xFFFFFFFFu, nulls, off);
        bad += __shfl_down_sync(0xFFFFFFFFu, bad, off);
        csum ^= __shfl_down_sync(0xFFFFFFFFu, csum, off);
    }
    if((threadIdx.x & 31u) == 0u)
    {
        atomicAdd(&stats[0], pairs);
        if(nulls)
            atomicAdd(&stats[1], nulls);
        if(bad)
            atomicAdd(&stats[2], bad);
        atomicXor(&stats[3], csum);
    }
}

/* ---------------------------------------------------------- fragmentation */

/* oc_frag_size of the oracle, on the device. */
__device__ __forceinline__ uint32_t frag_size(const mmc_frag_params& p, uint64_t i)
{
    const uint64_t m = mix64(p.seed, i, 0xF4A6ull);
    if(static_cast<uint32_t>(m % 1000u) < p.large_permille)
    {
        const double u = static_cast<double>((m >> 20) & 0xFFFFFFull) / 16777216.0;
        const double lo = static_cast<double>(p.large_lo), hi = static_cast<double>(p.large_hi);
        const uint32_t s = static_cast<uint32_t>(lo * exp(u * log(hi / lo)));
        return s < p.large_lo ? p.large_lo : (s > p.large_hi ? p.large_hi : s);
    }
    return p.small_lo + static_cast<uint32_t>((m >> 32) % static_cast<uint64_t>(p.small_hi - p.small_lo + 1u));
}

__device__ __forceinline__ uint64_t frag_tag(uint64_t slot, uint64_t off) { return (slot << 24) ^ off ^ 0xA5A5F00Dull; }

/* tags every 4 KiB and at the last aligned u64 of the block */
__device__ __forceinline__ void frag_write_tags(char* p, uint32_t size, uint64_t slot)
{
    for(uint32_t off = 0; off + 8u <= size; off += 4096u)
        *reinterpret_cast<uint64_t*>(p + off) = frag_tag(slot, off);
    const uint32_t last = (size & ~7u) - 8u;
    *reinterpret_cast<uint64_t*>(p + last) = frag_tag(slot, last);
}

__device__ __forceinline__ unsigned long long frag_check_tags(const char* p, uint32_t size, uint64_t slot)
{
    unsigned long long bad = 0;
    for(uint32_t off = 0; off + 8u <= size; off += 4096u)
        bad += *reinterpret_cast<const uint64_t*>(p + off) != frag_tag(slot, off);
    const uint32_t last = (size & ~7u) - 8u;
    bad += *reinterpret_cast<const uint64_t*>(p + last) != frag_tag(slot, last);
    return bad;
}

template<class Ids>
__global__ void __launch_bounds__(256) mmc_fill_kernel(mmc_device_handle h, mmc_frag_params p, uint64_t wave,
                                                       void** ptrs, uint32_t* sizes, uint64_t capacity,
                                                       unsigned long long* counters)
{
    if(dv::ld_rlx(reinterpret_cast<const uint32_t*>(&counters[4])) != 0u)
        return;
    const uint64_t T = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    const uint64_t t = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const uint32_t size = frag_size(p, p.first_request + wave * T + t);
    char* ptr = static_cast<char*>(dv::malloc<Ids>(h, size));
    atomicAdd(&counters[2], 1ull);
    if(ptr == nullptr)
    {
        atomicExch(reinterpret_cast<unsigned*>(&counters[4]), 1u);
        return;
    }
    const unsigned long long slot = atomicAdd(&counters[0], 1ull);
    if(slot >= capacity)
    {
        dv::free<Ids>(h, ptr);
        atomicExch(reinterpret_cast<unsigned*>(&counters[4]), 1u);
        return;
    }
    frag_write_tags(ptr, size, slot);
    ptrs[slot] = ptr;
    sizes[slot] = size;
    atomicAdd(&counters[1], static_cast<unsigned long long>(size));
}

template<class Ids>
__global__ void mmc_free_list_kernel(mmc_device_handle h, void** ptrs, uint32_t* sizes, const uint32_t* idx,
                                     uint64_t n, unsigned long long* counters)
{
    unsigned long long bytes = 0, bad = 0;
    for(uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
        i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        const uint32_t s = idx[i];
        char* ptr = static_cast<char*>(ptrs[s]);
        if(ptr == nullptr)
            continue;
        bad += frag_check_tags(ptr, sizes[s], s);
        bytes += sizes[s];
        dv::free<Ids>(h, ptr);
        ptrs[s] = nullptr;
        sizes[s] = 0u;
    }
    if(bytes)
        atomicAdd(&counters[1], 0ull - bytes);
    if(bad)
        atomicAdd(&counters[3], bad);
}

__global__ void mmc_verify_list_kernel(void* const* ptrs, const uint32_t* sizes, uint64_t n,
                                       unsigned long long* counters)
{
    unsigned long long bad = 0;
    for(uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
        i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        if(ptrs[i] != nullptr)
            bad += frag_check_tags(static_cast<const char*>(ptrs[i]), sizes[i], i);
    if(bad)
        atomicAdd(&counters[3], bad);
}

/* Verify workload: malloc(sizes[t]); write u32 (t ^ seed); optionally verify and free. */
template<bool ALLOC, bool FREE, class Ids>
__global__ void mmc_verify_kernel(mmc_device_handle h, uint32_t nthreads, const uint32_t* sizes, uint32_t seed,
                                  int64_t* offsets, unsigned long long* errors)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if(t >= nthreads)
        return;
    const uint32_t pattern = t ^ seed;
    const uint32_t words = dv::apply_padding(h.dataAlignment, sizes[t]) / 4u;
    uint32_t* p = nullptr;
    if(ALLOC)
    {
        p = static_cast<uint32_t*>(dv::malloc<Ids>(h, sizes[t]));
        offsets[t] = p ? static_cast<int64_t>(reinterpret_cast<char*>(p) - h.pages) : -1;
        if(p)
            for(uint32_t i = 0; i < sizes[t] / 4u; ++i)
                p[i] = pattern;
    }
    else
    {
        const int64_t off = offsets[t];
        p = off >= 0 ? reinterpret_cast<uint32_t*>(h.pages + off) : nullptr;
    }
    (void) words;
    if(FREE && p)
    {
        unsigned long long bad = 0;
        for(uint32_t i = 0; i < sizes[t] / 4u; ++i)
            bad += (p[i] != pattern);
        if(bad)
            atomicAdd(errors, bad);
        dv::free<Ids>(h, p);
    }
}

/* Relaxed device-scope atomicOr throughput (the roofline's denominator). */
__global__ void mmc_atomic_peak_kernel(uint32_t* buf, uint64_t mask, uint32_t iters, int returning, int contended,
                                       unsigned long long* sink)
{
    const uint64_t tid = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const uint64_t key = contended ? (tid >> 5) : tid;
    uint64_t x = mix64(0x5eedull, key, 0);
    uint32_t acc = 0;
    for(uint32_t i = 0; i < iters; ++i)
    {
        x = x * 6364136223846793005ull + 1442695040888963407ull;
        const uint64_t idx = (x >> 20) & mask;
        const uint32_t bit = 1u << ((x >> 7) & 31u);
        if(returning)
            acc += atomicOr(buf + idx, bit);
        else
            atomicOr(buf + idx, bit);
    }
    if(returning && acc == 0x9E3779B9u)
        atomicAdd(sink, 1ull);
}

extern "C" {

mmc_status mmc_run_program(mmc_heap* heap, const uint8_t* kinds, const uint64_t* args, int64_t n, int64_t* out,
                           void* stream)
{
    if(heap == nullptr || kinds == nullptr || args == nullptr || out == nullptr || n < 0)
        return fail(MMC_ERR_ARG, "null argument");
    mmc_device_handle h;
    mmc_heap_device_handle(heap, &h);
    cudaStream_t s = as_stream(stream);
    /* the 's' ops (host-side getAvailableSlots) split the program into kernels */
    uint8_t* hk = nullptr;
    if(cudaMallocHost(reinterpret_cast<void**>(&hk), n > 0 ? n : 1) != cudaSuccess)
        return fail(MMC_ERR_OOM, "pinned allocation failed");
    uint64_t* ha = nullptr;
    if(cudaMallocHost(reinterpret_cast<void**>(&ha), 8 * (n > 0 ? n : 1)) != cudaSuccess)
    {
        cudaFreeHost(hk);
        return fail(MMC_ERR_OOM, "pinned allocation failed");
    }
    mmc_status st = cuda_check(cudaMemcpyAsync(hk, kinds, n, cudaMemcpyDeviceToHost, s), "copy program kinds");
    if(st == MMC_OK)
        st = cuda_check(cudaMemcpyAsync(ha, args, 8 * n, cudaMemcpyDeviceToHost, s), "copy program args");
    if(st == MMC_OK)
        st = cuda_check(cudaStreamSynchronize(s), "wait for program");
    int64_t begin = 0;
    for(int64_t i = 0; st == MMC_OK && i <= n; ++i)
    {
        if(i == n || hk[i] == 's')
        {
            if(i > begin)
            {
                mmc_program_kernel<<<1, 1, 0, s>>>(h, kinds, args, begin, i, out);
                st = cuda_check(cudaGetLastError(), "program kernel");
            }
            if(st == MMC_OK && i < n)
            {
                const uint32_t slot = dv::apply_padding(h.dataAlignment, static_cast<uint32_t>(ha[i]));
                st = launch_available_slots(heap, slot, s, slots_result_word(heap));
                if(st == MMC_OK)
                {
                    mmc_store_result_kernel<<<1, 1, 0, s>>>(slots_result_word(heap), out + i);
                    st = cuda_check(cudaGetLastError(), "store slot count");
                }
            }
            begin = i + 1;
        }
    }
    if(st == MMC_OK)
        st = cuda_check(cudaStreamSynchronize(s), "wait for program kernels");
    cudaFreeHost(hk);
    cudaFreeHost(ha);
    return st;
}

mmc_status mmc_run_stress(mmc_heap* heap, const mmc_stress_params* p, const uint16_t* sizes,
                          unsigned long long* stats, void* stream)
{
    mmc::host::NvtxRange nvtx_range("mmc_run_stress");
    if(heap == nullptr || p == nullptr || stats == nullptr)
        return fail(MMC_ERR_ARG, "null argument");
    if(p->blocks == 0u || p->threads_per_block == 0u || p->threads_per_block > 256u || p->step == 0u
       || p->hi < p->lo || (p->write_pattern != MMC_PATTERN_THREAD && p->write_pattern != MMC_PATTERN_WARP)
       || (p->write_pattern == MMC_PATTERN_WARP && (p->threads_per_block % 32u) != 0u))
        return fail(MMC_ERR_ARG, "bad stress parameters");
    /* the kernel counts threads and each warp's pairs in 32 bits */
    if(static_cast<uint64_t>(p->blocks) * p->threads_per_block > 0xFFFFFFFFull || p->rounds > (1u << 26))
        return fail(MMC_ERR_ARG, "stress grid above 2^32 threads or more than 2^26 rounds");
    mmc_device_handle h;
    mmc_heap_device_handle(heap, &h);
    /* One instantiation per pattern mode: only the mode's code is in the
     * kernel. It keeps the multi-page path even when hi fits a page: built
     * without it (SmallRequests) the uniform stress measured 1.5 % slower on
     * GB300, from a different allocation of its 64 registers. */
    MMC_DISPATCH_IDS(h, if(p->write_pattern == MMC_PATTERN_WARP) mmc_stress_kernel<MMC_PATTERN_WARP, Ids>
                            <<<p->blocks, p->threads_per_block, 0, as_stream(stream)>>>(h, *p, sizes, stats);
                     else mmc_stress_kernel<MMC_PATTERN_THREAD, Ids>
                         <<<p->blocks, p->threads_per_block, 0, as_stream(stream)>>>(h, *p, sizes, stats));
    return cuda_check(cudaGetLastError(), "stress kernel");
}

mmc_status mmc_oldmalloc_set_heap(size_t bytes, int device)
{
    mmc_status st = cuda_check(cudaSetDevice(device), "cudaSetDevice");
    if(st == MMC_OK)
        st = cuda_check(cudaDeviceSetLimit(cudaLimitMallocHeapSize, bytes), "cudaDeviceSetLimit(MallocHeapSize)");
    if(st != MMC_OK)
        cudaGetLastError(); /* CUDA refuses the limit after ::malloc ran; do not leave the error pending
                               (CudaSetLimits.hpp:66-72 clears it the same way) */
    return st;
}

mmc_status mmc_run_stress_oldmalloc(const mmc_stress_params* p, const uint16_t* sizes, unsigned long long* stats,
                                    void* stream)
{
    if(p == nullptr || stats == nullptr)
        return fail(MMC_ERR_ARG, "null argument");
    if(p->blocks == 0u || p->threads_per_block == 0u || p->threads_per_block > 256u || p->step == 0u
       || p->hi < p->lo || (p->write_pattern == MMC_PATTERN_WARP && (p->threads_per_block % 32u) != 0u))
        return fail(MMC_ERR_ARG, "bad stress parameters");
    mmc_stress_oldmalloc_kernel<<<p->blocks, p->threads_per_block, 0, as_stream(stream)>>>(*p, sizes, stats);
    return cuda_check(cudaGetLastError(), "OldMalloc stress kernel");
}

mmc_status mmc_run_verify(mmc_heap* heap, uint32_t blocks, uint32_t tpb, const uint32_t* sizes, uint32_t seed,
                          int64_t* offsets, unsigned long long* errors, void* stream)
{
    if(heap == nullptr || sizes == nullptr || offsets == nullptr || errors == nullptr || blocks == 0u || tpb == 0u)
        return fail(MMC_ERR_ARG, "bad argument");
    mmc_device_handle h;
    mmc_heap_device_handle(heap, &h);
    MMC_DISPATCH_IDS(h, mmc_verify_kernel<true, true, Ids>
                     <<<blocks, tpb, 0, as_stream(stream)>>>(h, blocks * tpb, sizes, seed, offsets, errors));
    return cuda_check(cudaGetLastError(), "verify kernel");
}

mmc_status mmc_run_alloc_offsets(mmc_heap* heap, uint32_t blocks, uint32_t tpb, const uint32_t* sizes, uint32_t seed,
                                 int64_t* offsets, void* stream)
{
    if(heap == nullptr || sizes == nullptr || offsets == nullptr || blocks == 0u || tpb == 0u)
        return fail(MMC_ERR_ARG, "bad argument");
    mmc_device_handle h;
    mmc_heap_device_handle(heap, &h);
    MMC_DISPATCH_IDS(h, mmc_verify_kernel<true, false, Ids>
                     <<<blocks, tpb, 0, as_stream(stream)>>>(h, blocks * tpb, sizes, seed, offsets, nullptr));
    return cuda_check(cudaGetLastError(), "alloc kernel");
}

mmc_status mmc_run_free_offsets(mmc_heap* heap, uint32_t blocks, uint32_t tpb, const uint32_t* sizes, uint32_t seed,
                                const int64_t* offsets, unsigned long long* errors, void* stream)
{
    if(heap == nullptr || sizes == nullptr || offsets == nullptr || errors == nullptr || blocks == 0u || tpb == 0u)
        return fail(MMC_ERR_ARG, "bad argument");
    mmc_device_handle h;
    mmc_heap_device_handle(heap, &h);
    MMC_DISPATCH_IDS(h, mmc_verify_kernel<false, true, Ids><<<blocks, tpb, 0, as_stream(stream)>>>(
                            h, blocks * tpb, sizes, seed, const_cast<int64_t*>(offsets), errors));
    return cuda_check(cudaGetLastError(), "free kernel");
}

mmc_status mmc_run_fill(mmc_heap* heap, const mmc_frag_params* p, void** ptrs, uint32_t* sizes, uint64_t capacity,
                        unsigned long long* counters, void* stream)
{
    mmc::host::NvtxRange nvtx_range("mmc_run_fill");
    if(heap == nullptr || p == nullptr || ptrs == nullptr || sizes == nullptr || counters == nullptr)
        return fail(MMC_ERR_ARG, "null argument");
    if(p->blocks == 0u || p->threads_per_block == 0u || p->threads_per_block > 256u || p->small_lo < 8u
       || p->small_hi < p->small_lo || p->large_lo < 8u || p->large_hi < p->large_lo || p->large_permille > 1000u)
        return fail(MMC_ERR_ARG, "bad fragmentation parameters");
    mmc_device_handle h;
    mmc_heap_device_handle(heap, &h);
    for(uint32_t w = 0; w < p->waves; ++w)
    {
        MMC_DISPATCH_IDS(h, mmc_fill_kernel<Ids><<<p->blocks, p->threads_per_block, 0, as_stream(stream)>>>(
                                h, *p, w, ptrs, sizes, capacity, counters));
        const cudaError_t e = cudaGetLastError();
        if(e != cudaSuccess)
            return cuda_check(e, "fill kernel");
    }
    return MMC_OK;
}

mmc_status mmc_run_free_list(mmc_heap* heap, void** ptrs, uint32_t* sizes, const uint32_t* idx, uint64_t n,
                             unsigned long long* counters, void* stream)
{
    mmc::host::NvtxRange nvtx_range("mmc_run_free_list");
    if(heap == nullptr || ptrs == nullptr || sizes == nullptr || idx == nullptr || counters == nullptr)
        return fail(MMC_ERR_ARG, "null argument");
    if(n == 0u)
        return MMC_OK;
    mmc_device_handle h;
    mmc_heap_device_handle(heap, &h);
    const unsigned grid = static_cast<unsigned>(std::min<uint64_t>((n + 255u) / 256u, scan_grid(0) * 4u));
    MMC_DISPATCH_IDS(h, mmc_free_list_kernel<Ids><<<grid, 256, 0, as_stream(stream)>>>(h, ptrs, sizes, idx, n, counters));
    return cuda_check(cudaGetLastError(), "free-list kernel");
}

mmc_status mmc_run_verify_list(mmc_heap* heap, void* const* ptrs, const uint32_t* sizes, uint64_t n,
                               unsigned long long* counters, void* stream)
{
    if(heap == nullptr || ptrs == nullptr || sizes == nullptr || counters == nullptr)
        return fail(MMC_ERR_ARG, "null argument");
    if(n == 0u)
        return MMC_OK;
    const unsigned grid = static_cast<unsigned>(std::min<uint64_t>((n + 255u) / 256u, scan_grid(0) * 4u));
    mmc_verify_list_kernel<<<grid, 256, 0, as_stream(stream)>>>(ptrs, sizes, n, counters);
    return cuda_check(cudaGetLastError(), "verify-list kernel");
}

mmc_status mmc_atomic_peak(uint32_t* buf, uint64_t words, uint32_t blocks, uint32_t tpb, uint32_t iters,
                           int returning, int contended, unsigned long long* sink, void* stream)
{
    if(buf == nullptr || sink == nullptr || words == 0u || (words & (words - 1u)) != 0u || blocks == 0u || tpb == 0u)
        return fail(MMC_ERR_ARG, "words must be a power of two; buffers non-null");
    mmc_atomic_peak_kernel<<<blocks, tpb, 0, as_stream(stream)>>>(buf, words - 1u, iters, returning, contended,
                                                                  sink);
    return cuda_check(cudaGetLastError(), "atomic peak kernel");
}

} /* extern "C" */

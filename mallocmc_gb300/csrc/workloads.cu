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

/* Write then verify the u64 pattern m + i of `bytes` bytes at every lane's
 * block, cooperatively: the warp walks the blocks of its lanes in turn and
 * moves 512 contiguous bytes per instruction (16 per lane), instead of each
 * lane streaming its own block 16 bytes at a time across 32 cache lines.
 * Every lane of the warp must call it (blocks of lanes whose ptr is null are
 * skipped). Returns the pattern mismatches found in this lane's share. */
__device__ __forceinline__ unsigned long long warp_pattern(char* ptr, uint32_t bytes, uint64_t m,
                                                           unsigned long long& csum)
{
    const uint32_t lane = threadIdx.x & 31u;
    unsigned long long bad = 0;
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
    for(unsigned rest = have; rest != 0u; rest &= rest - 1u)
    {
        const int k = __ffs(static_cast<int>(rest)) - 1;
        const ulonglong2* q
            = reinterpret_cast<const ulonglong2*>(__shfl_sync(0xFFFFFFFFu, reinterpret_cast<unsigned long long>(ptr), k));
        const uint32_t n16 = __shfl_sync(0xFFFFFFFFu, bytes, k) / 16u;
        const uint64_t mk = __shfl_sync(0xFFFFFFFFu, m, k);
        for(uint32_t i = lane; i < n16; i += 32u)
        {
            const ulonglong2 v = q[i];
            bad += (v.x != mk + 2u * i) + (v.y != mk + 2u * i + 1u);
            csum += v.x ^ v.y;
        }
    }
    __syncwarp();
    return bad;
}

/* Uniform stress: sizes[r * nthreads + t] or drawn from the seed. */
__global__ void __launch_bounds__(256) mmc_stress_kernel(mmc_device_handle h, mmc_stress_params p,
                                                         const uint16_t* sizes, unsigned long long* stats)
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
        char* ptr = static_cast<char*>(dv::malloc<dv::GpuIds>(h, bytes));
        if(p.write_pattern == MMC_PATTERN_WARP)
        {
            /* every lane takes part, with or without a block */
            bad += warp_pattern(ptr, bytes, m, csum);
            if(ptr == nullptr)
                ++nulls;
            else
            {
                dv::free<dv::GpuIds>(h, ptr);
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
        dv::free<dv::GpuIds>(h, ptr);
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
        atomicAdd(&stats[0], pairs);
        if(nulls)
            atomicAdd(&stats[1], nulls);
        if(bad)
            atomicAdd(&stats[2], bad);
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

/* Verify workload: malloc(sizes[t]); write u32 (t ^ seed); optionally verify and free. */
template<bool ALLOC, bool FREE>
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
        p = static_cast<uint32_t*>(dv::malloc<dv::GpuIds>(h, sizes[t]));
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
        dv::free<dv::GpuIds>(h, p);
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
    if(heap == nullptr || p == nullptr || stats == nullptr)
        return fail(MMC_ERR_ARG, "null argument");
    if(p->blocks == 0u || p->threads_per_block == 0u || p->threads_per_block > 256u || p->step == 0u
       || p->hi < p->lo || (p->write_pattern != MMC_PATTERN_THREAD && p->write_pattern != MMC_PATTERN_WARP)
       || (p->write_pattern != MMC_PATTERN_THREAD && p->write_pattern != MMC_PATTERN_WARP)
       || (p->write_pattern == MMC_PATTERN_WARP && (p->threads_per_block % 32u) != 0u))
        return fail(MMC_ERR_ARG, "bad stress parameters");
    mmc_device_handle h;
    mmc_heap_device_handle(heap, &h);
    mmc_stress_kernel<<<p->blocks, p->threads_per_block, 0, as_stream(stream)>>>(h, *p, sizes, stats);
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
    mmc_verify_kernel<true, true><<<blocks, tpb, 0, as_stream(stream)>>>(h, blocks * tpb, sizes, seed, offsets,
                                                                       errors);
    return cuda_check(cudaGetLastError(), "verify kernel");
}

mmc_status mmc_run_alloc_offsets(mmc_heap* heap, uint32_t blocks, uint32_t tpb, const uint32_t* sizes, uint32_t seed,
                                 int64_t* offsets, void* stream)
{
    if(heap == nullptr || sizes == nullptr || offsets == nullptr || blocks == 0u || tpb == 0u)
        return fail(MMC_ERR_ARG, "bad argument");
    mmc_device_handle h;
    mmc_heap_device_handle(heap, &h);
    mmc_verify_kernel<true, false><<<blocks, tpb, 0, as_stream(stream)>>>(h, blocks * tpb, sizes, seed, offsets,
                                                                        nullptr);
    return cuda_check(cudaGetLastError(), "alloc kernel");
}

mmc_status mmc_run_free_offsets(mmc_heap* heap, uint32_t blocks, uint32_t tpb, const uint32_t* sizes, uint32_t seed,
                                const int64_t* offsets, unsigned long long* errors, void* stream)
{
    if(heap == nullptr || sizes == nullptr || offsets == nullptr || errors == nullptr || blocks == 0u || tpb == 0u)
        return fail(MMC_ERR_ARG, "bad argument");
    mmc_device_handle h;
    mmc_heap_device_handle(heap, &h);
    mmc_verify_kernel<false, true><<<blocks, tpb, 0, as_stream(stream)>>>(h, blocks * tpb, sizes, seed,
                                                                        const_cast<int64_t*>(offsets), errors);
    return cuda_check(cudaGetLastError(), "free kernel");
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

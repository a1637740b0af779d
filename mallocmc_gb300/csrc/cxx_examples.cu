/* cxx_examples.cu — user-side code written against the C++ drop-in API
 * (include/mallocMC/mallocMC.hpp), as the reference's examples are:
 *   example01  arrays of arrays allocated in kernels, vector addition, sums
 *              (reference: examples/mallocMC_example01.cpp)
 *   example03  device-side getAvailableSlots next to a live allocation
 *              (reference: examples/mallocMC_example03.cpp)
 * Built into libmallocmc_examples.so (linked against libmallocmc_gb300.so) and
 * driven by tests/test_cxx_api.py through the extern "C" wrappers below.
 *
 * Both reference examples construct a 1 GB heap with the default 2 GiB access
 * block; the reference divides by zero for that configuration
 * (Scatter.hpp:991-993). Here the same construction throws
 * std::invalid_argument, which mmcx_bad_config reports, and the examples run
 * with a 256 MiB access block.
 */
#include "mallocMC/mallocMC.hpp"

#include <cstdio>
#include <stdexcept>
#include <vector>

namespace
{
    struct ScatterHeapConfig
    {
        static constexpr auto pagesize = 4096;
        static constexpr auto accessblocksize = 256u * 1024u * 1024u;
        static constexpr auto regionsize = 16;
        static constexpr auto wastefactor = 2;
        static constexpr auto resetfreedpages = false;
    };
    struct ScatterHashConfig
    {
        static constexpr auto hashingK = 38183;
        static constexpr auto hashingDistMP = 17497;
        static constexpr auto hashingDistWP = 1;
        static constexpr auto hashingDistWPRel = 1;
    };
    struct ShrinkConfig
    {
        static constexpr auto dataAlignment = 16;
    };
    using Acc = mallocMC::AccGpuCuda;

    using ScatterAllocator = mallocMC::Allocator<
        Acc,
        mallocMC::CreationPolicies::Scatter<ScatterHeapConfig, ScatterHashConfig>,
        mallocMC::DistributionPolicies::Noop,
        mallocMC::OOMPolicies::ReturnNull,
        mallocMC::ReservePoolPolicies::AlpakaBuf<Acc>,
        mallocMC::AlignmentPolicies::Shrink<ShrinkConfig>>;

    using DefaultAllocator = mallocMC::Allocator<
        Acc,
        mallocMC::CreationPolicies::Scatter<>,
        mallocMC::DistributionPolicies::XMallocSIMD<>,
        mallocMC::OOMPolicies::ReturnNull,
        mallocMC::ReservePoolPolicies::AlpakaBuf<Acc>,
        mallocMC::AlignmentPolicies::Shrink<>>;

    using OldAllocator = mallocMC::Allocator<
        Acc,
        mallocMC::CreationPolicies::OldMalloc,
        mallocMC::DistributionPolicies::Noop,
        mallocMC::OOMPolicies::ReturnNull,
        mallocMC::ReservePoolPolicies::CudaSetLimits,
        mallocMC::AlignmentPolicies::Noop>;

    /* The reference's policy matrix (tests/policies.cpp:83-187): Scatter or
     * OldMalloc x XMallocSIMD or Noop x Shrink or Noop, each with its reserve
     * pool and ReturnNull; there one thread mallocs 4000 bytes and frees them. */
    template<class Creation, class Distribution, class ReservePool, class Alignment>
    using PolicyAllocator = mallocMC::Allocator<Acc, Creation, Distribution, mallocMC::OOMPolicies::ReturnNull,
                                                ReservePool, Alignment>;
    using Sc = mallocMC::CreationPolicies::Scatter<ScatterHeapConfig, ScatterHashConfig>;
    using Om = mallocMC::CreationPolicies::OldMalloc;
    using Xm = mallocMC::DistributionPolicies::XMallocSIMD<>;
    using Nd = mallocMC::DistributionPolicies::Noop;
    using Ab = mallocMC::ReservePoolPolicies::AlpakaBuf<Acc>;
    using Cl = mallocMC::ReservePoolPolicies::CudaSetLimits;
    using Sh = mallocMC::AlignmentPolicies::Shrink<ShrinkConfig>;
    using Na = mallocMC::AlignmentPolicies::Noop;

    template<class A>
    __global__ void policyMatrixKernel(typename A::AllocatorHandle h, int* ok)
    {
        const Acc acc{};
        void* p = h.malloc(acc, 4000);
        if(p != nullptr)
        {
            h.free(acc, p);
            *ok = 1;
        }
    }

    template<class A>
    std::string policy_info()
    {
        return A::info("\n");
    }

    __global__ void oldMallocKernel(OldAllocator::AllocatorHandle h, int length, unsigned long long* sums, int* fails)
    {
        const Acc acc{};
        const unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
        int* a = static_cast<int*>(h.malloc(acc, length * sizeof(int)));
        if(a == nullptr)
        {
            atomicAdd(fails, 1);
            sums[id] = 0;
            return;
        }
        unsigned long long s = 0;
        for(int i = 0; i < length; ++i)
            a[i] = static_cast<int>(id * length + i);
        for(int i = 0; i < length; ++i)
            s += static_cast<unsigned long long>(a[i]);
        sums[id] = s;
        if(h.getAvailableSlots(acc, 16) != 0u)
            atomicAdd(fails, 1000); /* OldMalloc provides no count: must be 0 */
        h.free(acc, a);
    }

    __device__ int** arA;
    __device__ int** arB;
    __device__ int** arC;
    __device__ int* ar3;

    __global__ void createArrayPointers(int x, int y, ScatterAllocator::AllocatorHandle h)
    {
        const Acc acc{};
        arA = static_cast<int**>(h.malloc(acc, sizeof(int*) * x * y));
        arB = static_cast<int**>(h.malloc(acc, sizeof(int*) * x * y));
        arC = static_cast<int**>(h.malloc(acc, sizeof(int*) * x * y));
    }

    __global__ void fillArrays(int length, ScatterAllocator::AllocatorHandle h, int* failures)
    {
        const Acc acc{};
        const unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
        arA[id] = static_cast<int*>(h.malloc(acc, length * sizeof(int)));
        arB[id] = static_cast<int*>(h.malloc(acc, length * sizeof(int)));
        arC[id] = static_cast<int*>(h.malloc(acc, length * sizeof(int)));
        if(!arA[id] || !arB[id] || !arC[id])
        {
            atomicAdd(failures, 1);
            return;
        }
        for(int i = 0; i < length; ++i)
        {
            arA[id][i] = static_cast<int>(id * length + i);
            arB[id][i] = static_cast<int>(id * length + i);
        }
    }

    __global__ void addArrays(int length, unsigned long long* sums)
    {
        const unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
        unsigned long long s = 0;
        if(arA[id] && arB[id] && arC[id])
            for(int i = 0; i < length; ++i)
            {
                arC[id][i] = arA[id][i] + arB[id][i];
                s += static_cast<unsigned long long>(arC[id][i]);
            }
        sums[id] = s;
    }

    __global__ void freeArrays(ScatterAllocator::AllocatorHandle h)
    {
        const unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
        h.free(arA[id]);
        h.free(arB[id]);
        h.free(arC[id]);
    }

    __global__ void freeArrayPointers(ScatterAllocator::AllocatorHandle h)
    {
        h.free(arA);
        h.free(arB);
        h.free(arC);
    }

    __global__ void example03Kernel(ScatterAllocator::AllocatorHandle h, unsigned* slots, int* values)
    {
        const Acc acc{};
        const unsigned id = threadIdx.x;
        if(id == 0)
            ar3 = static_cast<int*>(h.malloc(acc, sizeof(int) * 32));
        __syncthreads();
        slots[id] = h.getAvailableSlots(acc, 1);
        if(ar3 != nullptr)
        {
            ar3[id] = static_cast<int>(id);
            values[id] = ar3[id];
        }
        __syncthreads();
        if(id == 0)
            h.free(acc, ar3);
    }

    /* User code on the raw device API whose requests fit a page: the kernel
     * is built with SmallRequests, which leaves the multi-page search out of
     * it. Here one request above a page is made on purpose: it fails
     * (nullptr, MMC_DEVERR_PAGEBASED), while the same request through the
     * handle takes the multi-page path. */
    __global__ void smallRequestsKernel(ScatterAllocator::AllocatorHandle h, int* out)
    {
        using Small = mmc::dev::SmallRequests<ScatterAllocator::AllocatorHandle::Ids>;
        void* a = mmc::dev::malloc<Small>(h.devAllocator, 256);
        void* b = mmc::dev::malloc<Small>(h.devAllocator, 3 * 4096 + 16);
        void* c = h.malloc(3 * 4096 + 16);
        out[0] = a != nullptr;
        out[1] = b == nullptr;
        out[2] = c != nullptr;
        if(a != nullptr)
            mmc::dev::free<Small>(h.devAllocator, a);
        if(c != nullptr)
            h.free(c);
    }

    int report(const std::exception& e)
    {
        std::fprintf(stderr, "mmcx: %s\n", e.what());
        return 1;
    }
} // namespace

extern "C" {

/* example01: returns 0 on success; *sum is the GPU sum of C = A + B over all
 * threads, *gaussian the closed form n(n-1) with n = threads * length,
 * *slots_1mib the host getAvailableSlots(1 MiB) before freeing. */
int mmcx_example01(int device, int length, unsigned long long* sum, unsigned long long* gaussian,
                   unsigned* slots_1mib, int* failures)
{
    try
    {
        cudaSetDevice(device);
        const unsigned block = 32;
        const unsigned grid = (length + block - 1) / block;
        ScatterAllocator alloc(device, nullptr, 1U * 1024U * 1024U * 1024U);
        int* d_fail = nullptr;
        unsigned long long* d_sums = nullptr;
        cudaMalloc(&d_fail, sizeof(int));
        cudaMemset(d_fail, 0, sizeof(int));
        cudaMalloc(&d_sums, sizeof(unsigned long long) * block * grid);
        createArrayPointers<<<1, 1>>>(grid, block, alloc.getAllocatorHandle());
        fillArrays<<<grid, block>>>(length, alloc.getAllocatorHandle(), d_fail);
        addArrays<<<grid, block>>>(length, d_sums);
        std::vector<unsigned long long> h(block * grid);
        cudaMemcpy(h.data(), d_sums, sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost);
        cudaMemcpy(failures, d_fail, sizeof(int), cudaMemcpyDeviceToHost);
        unsigned long long s = 0;
        for(auto v : h)
            s += v;
        *sum = s;
        const unsigned long long n = static_cast<unsigned long long>(block) * grid * length;
        *gaussian = n * (n - 1);
        if(mallocMC::Traits<ScatterAllocator>::providesAvailableSlots)
            *slots_1mib = alloc.getAvailableSlots(device, nullptr, 1024U * 1024U);
        freeArrays<<<grid, block>>>(alloc.getAllocatorHandle());
        freeArrayPointers<<<1, 1>>>(alloc.getAllocatorHandle());
        const cudaError_t e = cudaDeviceSynchronize();
        cudaFree(d_fail);
        cudaFree(d_sums);
        return e == cudaSuccess ? 0 : 2;
    }
    catch(const std::exception& e)
    {
        return report(e);
    }
}

/* example03: 32 threads of one block; slots[32] are the device-side counts of
 * 1-byte slots seen while thread 0's 128-byte block is live, values[32] what
 * each thread stored into it, *host_slots the host count after the free. */
int mmcx_example03(int device, unsigned* slots, int* values, unsigned* host_slots)
{
    try
    {
        cudaSetDevice(device);
        ScatterAllocator alloc(device, nullptr, 1U * 1024U * 1024U * 1024U);
        unsigned* d_slots = nullptr;
        int* d_values = nullptr;
        cudaMalloc(&d_slots, 32 * sizeof(unsigned));
        cudaMalloc(&d_values, 32 * sizeof(int));
        example03Kernel<<<1, 32>>>(alloc.getAllocatorHandle(), d_slots, d_values);
        cudaMemcpy(slots, d_slots, 32 * sizeof(unsigned), cudaMemcpyDeviceToHost);
        cudaMemcpy(values, d_values, 32 * sizeof(int), cudaMemcpyDeviceToHost);
        *host_slots = alloc.getAvailableSlots(device, nullptr, 1);
        cudaFree(d_slots);
        cudaFree(d_values);
        return cudaDeviceSynchronize() == cudaSuccess ? 0 : 2;
    }
    catch(const std::exception& e)
    {
        return report(e);
    }
}

/* The reference examples' configuration (1 GB heap, default 2 GiB access
 * block): returns 1 if construction throws std::invalid_argument, else 0.
 * No device work happens before the check. */
int mmcx_bad_config(int device)
{
    try
    {
        DefaultAllocator alloc(device, nullptr, 1U * 1024U * 1024U * 1024U);
        return 0;
    }
    catch(const std::invalid_argument&)
    {
        return 1;
    }
}

/* The same policy API over CUDA's own device heap (CreationPolicies::OldMalloc
 * with ReservePoolPolicies::CudaSetLimits): *sum over threads of their array
 * sums, *gaussian the closed form n(n-1)/2, host slot count (0: no count). */
int mmcx_oldmalloc(int device, int length, unsigned long long* sum, unsigned long long* gaussian, unsigned* slots,
                   int* failures)
{
    try
    {
        cudaSetDevice(device);
        OldAllocator alloc(device, nullptr, 64U * 1024U * 1024U);
        const unsigned block = 64, grid = 8;
        int* d_fail = nullptr;
        unsigned long long* d_sums = nullptr;
        cudaMalloc(&d_fail, sizeof(int));
        cudaMemset(d_fail, 0, sizeof(int));
        cudaMalloc(&d_sums, sizeof(unsigned long long) * block * grid);
        oldMallocKernel<<<grid, block>>>(alloc.getAllocatorHandle(), length, d_sums, d_fail);
        std::vector<unsigned long long> h(block * grid);
        cudaMemcpy(h.data(), d_sums, sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost);
        cudaMemcpy(failures, d_fail, sizeof(int), cudaMemcpyDeviceToHost);
        unsigned long long s = 0;
        for(auto v : h)
            s += v;
        *sum = s;
        const unsigned long long n = static_cast<unsigned long long>(block) * grid * length;
        *gaussian = n * (n - 1) / 2;
        *slots = alloc.getAvailableSlots(device, nullptr, 16);
        const cudaError_t e = cudaDeviceSynchronize();
        cudaFree(d_fail);
        cudaFree(d_sums);
        return e == cudaSuccess ? 0 : 2;
    }
    catch(const std::exception& e)
    {
        return report(e);
    }
}

/* SmallRequests: out[3] = {the small request succeeded, the request above a
 * page failed, the same request through the handle succeeded}; *flags the
 * heap's device error bits afterwards. */
int mmcx_small_requests(int device, int* out, unsigned* flags)
{
    try
    {
        cudaSetDevice(device);
        ScatterAllocator alloc(device, nullptr, 1U * 1024U * 1024U * 1024U);
        int* d_out = nullptr;
        cudaMalloc(&d_out, 3 * sizeof(int));
        smallRequestsKernel<<<1, 1>>>(alloc.getAllocatorHandle(), d_out);
        cudaMemcpy(out, d_out, 3 * sizeof(int), cudaMemcpyDeviceToHost);
        *flags = alloc.errorFlags();
        cudaFree(d_out);
        return cudaDeviceSynchronize() == cudaSuccess ? 0 : 2;
    }
    catch(const std::exception& e)
    {
        return report(e);
    }
}

/* info() strings of the two allocator types (host only). */
/* The info() strings of the eight allocators of the reference's policy matrix,
 * separated by "--" lines (host only). */
int mmcx_policy_matrix_info(char* buf, size_t len)
{
    const std::string s = policy_info<PolicyAllocator<Sc, Xm, Ab, Sh>>() + "--\n"
                          + policy_info<PolicyAllocator<Sc, Xm, Ab, Na>>() + "--\n"
                          + policy_info<PolicyAllocator<Sc, Nd, Ab, Sh>>() + "--\n"
                          + policy_info<PolicyAllocator<Sc, Nd, Ab, Na>>() + "--\n"
                          + policy_info<PolicyAllocator<Om, Xm, Cl, Sh>>() + "--\n"
                          + policy_info<PolicyAllocator<Om, Xm, Cl, Na>>() + "--\n"
                          + policy_info<PolicyAllocator<Om, Nd, Cl, Sh>>() + "--\n"
                          + policy_info<PolicyAllocator<Om, Nd, Cl, Na>>();
    if(buf == nullptr || len == 0)
        return 1;
    std::snprintf(buf, len, "%s", s.c_str());
    return s.size() < len ? 0 : 1;
}

/* The device code of the same eight allocators, compiled: the host entry of
 * each one's malloc(4000)/free kernel (i in 0..7, in the order above). */
const void* mmcx_policy_matrix_kernel(int i)
{
    static const void* const k[8] = {
        reinterpret_cast<const void*>(&policyMatrixKernel<PolicyAllocator<Sc, Xm, Ab, Sh>>),
        reinterpret_cast<const void*>(&policyMatrixKernel<PolicyAllocator<Sc, Xm, Ab, Na>>),
        reinterpret_cast<const void*>(&policyMatrixKernel<PolicyAllocator<Sc, Nd, Ab, Sh>>),
        reinterpret_cast<const void*>(&policyMatrixKernel<PolicyAllocator<Sc, Nd, Ab, Na>>),
        reinterpret_cast<const void*>(&policyMatrixKernel<PolicyAllocator<Om, Xm, Cl, Sh>>),
        reinterpret_cast<const void*>(&policyMatrixKernel<PolicyAllocator<Om, Xm, Cl, Na>>),
        reinterpret_cast<const void*>(&policyMatrixKernel<PolicyAllocator<Om, Nd, Cl, Sh>>),
        reinterpret_cast<const void*>(&policyMatrixKernel<PolicyAllocator<Om, Nd, Cl, Na>>)};
    return (i >= 0 && i < 8) ? k[i] : nullptr;
}

int mmcx_info(char* buf, size_t len)
{
    const std::string s = ScatterAllocator::info("\n") + "--\n" + DefaultAllocator::info("\n");
    if(buf == nullptr || len == 0)
        return 1;
    const size_t n = std::min(len - 1, s.size());
    std::copy(s.begin(), s.begin() + static_cast<long>(n), buf);
    buf[n] = '\0';
    return 0;
}

} /* extern "C" */

/* mallocMC.hpp — the reference's C++ policy/handle API on the GB300 heap.
 *
 * Source compatible with code written against mallocMC 2.6
 * (src/include/mallocMC/mallocMC.hpp and the headers it includes):
 *
 *   using ScatterAllocator = mallocMC::Allocator<
 *       Acc,
 *       mallocMC::CreationPolicies::Scatter<HeapCfg, HashCfg>,
 *       mallocMC::DistributionPolicies::XMallocSIMD<XCfg>,
 *       mallocMC::OOMPolicies::ReturnNull,
 *       mallocMC::ReservePoolPolicies::AlpakaBuf<Acc>,
 *       mallocMC::AlignmentPolicies::Shrink<ShrinkCfg>>;
 *   ScatterAllocator alloc(dev, queue, bytes);
 *   kernel<<<g, b>>>(alloc.getAllocatorHandle());      // handle by value
 *   // in the kernel: p = handle.malloc(acc, n); handle.free(acc, p);
 *
 * Differences a caller sees: `dev` is a CUDA device ordinal and `queue` a
 * cudaStream_t (there is no alpaka layer); the Acc template parameter and the
 * `acc` argument of the device functions are accepted and ignored, and
 * overloads without `acc` exist. The heap itself lives behind the C ABI
 * (include/mallocmc_gb300.h, libmallocmc_gb300.so); the device functions are
 * inlined from scatter_device.cuh.
 */
#pragma once

#include "../mallocmc_gb300.h"
#include "scatter_device.cuh"

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

/* version.hpp:40-47 */
#define MALLOCMC_VERSION_MAJOR 2
#define MALLOCMC_VERSION_MINOR 6
#define MALLOCMC_VERSION_PATCH 0
#define MALLOCMC_FLAVOR "gb300"

namespace mallocMC
{
    /* Tag usable as the (ignored) accelerator type. */
    struct AccGpuCuda
    {
    };

    constexpr uint32_t maxThreadsPerBlock = 1024; /* mallocMC_utils.hpp:187 */

    namespace CreationPolicies
    {
        namespace ScatterConf
        {
            /* Scatter.hpp:56-78 */
            struct DefaultScatterConfig
            {
                static constexpr auto pagesize = 4096;
                static constexpr auto accessblocksize = 2u * 1024u * 1024u * 1024u;
                static constexpr auto regionsize = 16;
                static constexpr auto wastefactor = 2;
                static constexpr auto resetfreedpages = false;
            };
            /* Scatter.hpp:80-86 */
            struct DefaultScatterHashingParams
            {
                static constexpr auto hashingK = 38183;
                static constexpr auto hashingDistMP = 17497;
                static constexpr auto hashingDistWP = 1;
                static constexpr auto hashingDistWPRel = 1;
            };
        } // namespace ScatterConf

        /* Scatter<T_Config, T_Hashing> (Scatter.hpp:106-207). The -D overrides of
         * the reference (MALLOCMC_CP_SCATTER_*) keep their precedence. */
        template<class T_Config = ScatterConf::DefaultScatterConfig,
                 class T_Hashing = ScatterConf::DefaultScatterHashingParams>
        class Scatter
        {
        public:
            using HeapProperties = T_Config;
            using HashingProperties = T_Hashing;
            static constexpr bool providesAvailableSlots = true;
            static constexpr bool usesHeap = true;

#ifdef MALLOCMC_CP_SCATTER_PAGESIZE
            static constexpr uint32_t pagesize = MALLOCMC_CP_SCATTER_PAGESIZE;
#else
            static constexpr uint32_t pagesize = HeapProperties::pagesize;
#endif
#ifdef MALLOCMC_CP_SCATTER_ACCESSBLOCKSIZE
            static constexpr size_t accessblocksize = MALLOCMC_CP_SCATTER_ACCESSBLOCKSIZE;
#else
            static constexpr size_t accessblocksize = HeapProperties::accessblocksize;
#endif
#ifdef MALLOCMC_CP_SCATTER_REGIONSIZE
            static constexpr uint32_t regionsize = MALLOCMC_CP_SCATTER_REGIONSIZE;
#else
            static constexpr uint32_t regionsize = HeapProperties::regionsize;
#endif
#ifdef MALLOCMC_CP_SCATTER_WASTEFACTOR
            static constexpr uint32_t wastefactor = MALLOCMC_CP_SCATTER_WASTEFACTOR;
#else
            static constexpr uint32_t wastefactor = HeapProperties::wastefactor;
#endif
#ifdef MALLOCMC_CP_SCATTER_RESETFREEDPAGES
            static constexpr bool resetfreedpages = MALLOCMC_CP_SCATTER_RESETFREEDPAGES;
#else
            static constexpr bool resetfreedpages = HeapProperties::resetfreedpages;
#endif
#ifdef MALLOCMC_CP_SCATTER_HASHINGK
            static constexpr uint32_t hashingK = MALLOCMC_CP_SCATTER_HASHINGK;
#else
            static constexpr uint32_t hashingK = HashingProperties::hashingK;
#endif
#ifdef MALLOCMC_CP_SCATTER_HASHINGDISTMP
            static constexpr uint32_t hashingDistMP = MALLOCMC_CP_SCATTER_HASHINGDISTMP;
#else
            static constexpr uint32_t hashingDistMP = HashingProperties::hashingDistMP;
#endif
#ifdef MALLOCMC_CP_SCATTER_HASHINGDISTWP
            static constexpr uint32_t hashingDistWP = MALLOCMC_CP_SCATTER_HASHINGDISTWP;
#else
            static constexpr uint32_t hashingDistWP = HashingProperties::hashingDistWP;
#endif
#ifdef MALLOCMC_CP_SCATTER_HASHINGDISTWPREL
            static constexpr uint32_t hashingDistWPRel = MALLOCMC_CP_SCATTER_HASHINGDISTWPREL;
#else
            static constexpr uint32_t hashingDistWPRel = HashingProperties::hashingDistWPRel;
#endif
            static constexpr uint32_t _pagesize = pagesize;
            static constexpr size_t _accessblocksize = accessblocksize;
            static constexpr uint32_t _regionsize = regionsize;
            static constexpr uint32_t _wastefactor = wastefactor;
            static constexpr bool _resetfreedpages = resetfreedpages;

            static void fill(mmc_config& c)
            {
                c.pagesize = pagesize;
                c.accessblocksize = accessblocksize;
                c.regionsize = regionsize;
                c.wastefactor = wastefactor;
                c.resetfreedpages = resetfreedpages ? 1u : 0u;
                c.hashingK = hashingK;
                c.hashingDistMP = hashingDistMP;
                c.hashingDistWP = hashingDistWP;
                c.hashingDistWPRel = hashingDistWPRel;
            }

            /* Scatter.hpp:1354-1370 */
            static auto classname() -> std::string
            {
                std::stringstream ss;
                ss << "Scatter[pagesize=" << pagesize << ",accessblocksize=" << accessblocksize
                   << ",regionsize=" << regionsize << ",wastefactor=" << wastefactor
                   << ",resetfreedpages=" << resetfreedpages << ",minChunkSize=" << (pagesize - 128u) / 1024u
                   << ",HierarchyThreshold=" << (pagesize - 8u) / 33u << ",hashingK=" << hashingK
                   << ",hashingDistMP=" << hashingDistMP << ",hashingDistWP=" << hashingDistWP
                   << ",hashingDistWPRel=" << hashingDistWPRel << "]";
                return ss.str();
            }
        };
        /* OldMalloc (creationPolicies/OldMalloc.hpp:46-84): CUDA's own device
         * malloc/free; provides no slot count (:51). Pair it with
         * ReservePoolPolicies::CudaSetLimits. */
        class OldMalloc
        {
        public:
            static constexpr bool providesAvailableSlots = false;
            static constexpr bool usesHeap = false;
            static void fill(mmc_config&) {}
            static auto classname() -> std::string { return "OldMalloc"; }
        };
    } // namespace CreationPolicies

    namespace DistributionPolicies
    {
        namespace XMallocSIMDConf
        {
            struct DefaultXMallocConfig
            {
                static constexpr auto pagesize = 4096;
            };
        } // namespace XMallocSIMDConf

        /* XMallocSIMD<T_Config> (XMallocSIMD.hpp:76-185) */
        template<typename T_Config = XMallocSIMDConf::DefaultXMallocConfig>
        class XMallocSIMD
        {
        public:
            using Properties = T_Config;
#ifdef MALLOCMC_DP_XMALLOCSIMD_PAGESIZE
            static constexpr uint32_t pagesize = MALLOCMC_DP_XMALLOCSIMD_PAGESIZE;
#else
            static constexpr uint32_t pagesize = Properties::pagesize;
#endif
            static constexpr uint32_t _pagesize = pagesize;
            static constexpr uint32_t code = MMC_DIST_XMALLOCSIMD;
            static auto classname() -> std::string { return "XMallocSIMD[" + std::to_string(pagesize) + "]"; }
        };

        /* distributionPolicies/Noop.hpp:46-72 */
        class Noop
        {
        public:
            static constexpr uint32_t code = MMC_DIST_NOOP;
            static auto classname() -> std::string { return "Noop"; }
        };
    } // namespace DistributionPolicies

    namespace OOMPolicies
    {
        /* ReturnNull.hpp:44-57 */
        class ReturnNull
        {
        public:
            static constexpr uint32_t code = MMC_OOM_RETURNNULL;
            __host__ __device__ static auto handleOOM(void*) -> void* { return nullptr; }
            static auto classname() -> std::string { return "ReturnNull"; }
        };

        /* BadAllocException.hpp:50-74. The reference asserts on the device; here a
         * failed allocation sets MMC_DEVERR_OOM (see Allocator::errorFlags) and
         * returns nullptr, so no kernel traps. */
        class BadAllocException
        {
        public:
            static constexpr uint32_t code = MMC_OOM_FLAG;
            static auto classname() -> std::string { return "BadAllocException"; }
        };
    } // namespace OOMPolicies

    namespace ReservePoolPolicies
    {
        /* AlpakaBuf.hpp:38-61: the heap allocates its own pool (cudaMalloc). */
        template<typename AlpakaAcc = AccGpuCuda>
        struct AlpakaBuf
        {
            static auto classname() -> std::string { return "AlpakaBuf"; }
        };

        /* CudaSetLimits (CudaSetLimits.hpp:57-78): sizes CUDA's device heap for
         * OldMalloc through cudaLimitMallocHeapSize of the current context. */
        struct CudaSetLimits
        {
            static auto classname() -> std::string { return "CudaSetLimits"; }
        };
    } // namespace ReservePoolPolicies

    namespace AlignmentPolicies
    {
        namespace ShrinkConfig
        {
            struct DefaultShrinkConfig
            {
                static constexpr auto dataAlignment = 16;
            };
        } // namespace ShrinkConfig

        /* Shrink<T_Config> (Shrink.hpp:80-146) */
        template<typename T_Config = ShrinkConfig::DefaultShrinkConfig>
        class Shrink
        {
        public:
            using Properties = T_Config;
#ifdef MALLOCMC_AP_SHRINK_DATAALIGNMENT
            static constexpr size_t dataAlignment = MALLOCMC_AP_SHRINK_DATAALIGNMENT;
#else
            static constexpr size_t dataAlignment = Properties::dataAlignment;
#endif
            static_assert(dataAlignment != 0 && (dataAlignment & (dataAlignment - 1)) == 0,
                          "dataAlignment must also be a power of 2");
            __host__ __device__ static auto applyPadding(uint32_t bytes) -> uint32_t
            {
                return mmc::dev::apply_padding(static_cast<uint32_t>(dataAlignment), bytes);
            }
            static auto classname() -> std::string { return "Shrink[" + std::to_string(dataAlignment) + "]"; }
        };

        /* alignmentPolicies/Noop.hpp:47-65 */
        class Noop
        {
        public:
            static constexpr size_t dataAlignment = 1;
            __host__ __device__ static auto applyPadding(uint32_t bytes) -> uint32_t { return bytes; }
            static auto classname() -> std::string { return "Noop"; }
        };
    } // namespace AlignmentPolicies

    /* PolicyCheck2 (mallocMC_constraints.hpp:84-88) */
    template<typename C, typename D>
    struct PolicyCheck2
    {
        static constexpr bool ok = true;
    };
    template<typename X, typename Y, typename Z>
    struct PolicyCheck2<CreationPolicies::Scatter<X, Y>, DistributionPolicies::XMallocSIMD<Z>>
    {
        static_assert(CreationPolicies::Scatter<X, Y>::pagesize == DistributionPolicies::XMallocSIMD<Z>::pagesize,
                      "Pagesize must be the same when combining Scatter and XMallocSIMD");
        static constexpr bool ok = true;
    };

    /* HeapInfo (allocator.hpp:77-81) */
    struct HeapInfo
    {
        void* p;
        size_t size;
    };

    namespace detail
    {
        /* Scatter's resetfreedpages as 0/1; 0 for creation policies without one */
        template<typename T, typename = void>
        struct ResetOf
        {
            static constexpr uint32_t value = 0u;
        };
        template<typename T>
        struct ResetOf<T, std::void_t<decltype(T::resetfreedpages)>>
        {
            static constexpr uint32_t value = T::resetfreedpages ? 1u : 0u;
        };
    } // namespace detail

    /* AllocatorHandleImpl (mallocMC_allocator_handle.hpp:35-63): passed to
     * kernels by value; all heap constants ride in kernel parameter space. */
    template<typename T_HostAllocator>
    struct AllocatorHandleImpl
    {
        mmc_device_handle devAllocator;

        /* The thread ids with the allocator's policy values fixed at compile
         * time, as the reference's templates fix them: only the code of this
         * configuration is compiled into the user's kernels. */
        using Ids = mmc::dev::GpuIdsFixed<
            detail::ResetOf<typename T_HostAllocator::CreationPolicy>::value,
            T_HostAllocator::DistributionPolicy::code,
            T_HostAllocator::OOMPolicy::code,
            static_cast<uint32_t>(T_HostAllocator::AlignmentPolicy::dataAlignment)>;

        AllocatorHandleImpl() = default;
        explicit AllocatorHandleImpl(mmc_device_handle const& h) : devAllocator(h) {}

        __device__ auto malloc(size_t size) -> void*
        {
            if constexpr(T_HostAllocator::CreationPolicy::usesHeap)
                return mmc::dev::malloc<Ids>(devAllocator, size);
            else
                return ::malloc(static_cast<size_t>(static_cast<uint32_t>(size))); /* OldMalloc.hpp:56-60 */
        }
        template<typename AlpakaAcc>
        __device__ auto malloc(AlpakaAcc const&, size_t size) -> void*
        {
            return malloc(size);
        }

        __device__ void free(void* p)
        {
            if constexpr(T_HostAllocator::CreationPolicy::usesHeap)
                mmc::dev::free<Ids>(devAllocator, p);
            else
            {
                mmc::dev::release_fence(); /* the accesses before the free are performed first */
                ::free(p);                 /* OldMalloc.hpp:62-66 */
            }
        }
        template<typename AlpakaAcc>
        __device__ void free(AlpakaAcc const&, void* p)
        {
            free(p);
        }

        /* device_allocator.hpp:98-106 (0 when the creation policy provides no
         * count); any subset of a warp's threads may call it */
        __device__ auto getAvailableSlots(size_t slotSize) -> unsigned
        {
            if constexpr(T_HostAllocator::CreationPolicy::providesAvailableSlots)
                return mmc::dev::available_slots<Ids>(devAllocator, slotSize);
            else
                return 0u;
        }
        template<typename AlpakaAcc>
        __device__ auto getAvailableSlots(AlpakaAcc const&, size_t slotSize) -> unsigned
        {
            return getAvailableSlots(slotSize);
        }
    };

    namespace detail
    {
        inline void throw_status(mmc_status st, const char* what)
        {
            if(st == MMC_OK)
                return;
            std::string msg = std::string(what) + ": " + mmc_last_error();
            if(st == MMC_ERR_CONFIG || st == MMC_ERR_ARG)
                throw std::invalid_argument(msg);
            throw std::runtime_error(msg);
        }
    } // namespace detail

    /* Allocator (allocator.hpp:97-242) */
    template<typename AlpakaAcc, typename T_CreationPolicy, typename T_DistributionPolicy, typename T_OOMPolicy,
             typename T_ReservePoolPolicy, typename T_AlignmentPolicy>
    class Allocator
    {
        static_assert(PolicyCheck2<T_CreationPolicy, T_DistributionPolicy>::ok, "policy constraint");

    public:
        using CreationPolicy = T_CreationPolicy;
        using DistributionPolicy = T_DistributionPolicy;
        using OOMPolicy = T_OOMPolicy;
        using ReservePoolPolicy = T_ReservePoolPolicy;
        using AlignmentPolicy = T_AlignmentPolicy;
        using HeapInfoVector = std::vector<HeapInfo>;
        using AllocatorHandle = AllocatorHandleImpl<Allocator>;

        Allocator(Allocator const&) = delete;
        auto operator=(Allocator const&) -> Allocator& = delete;

        /* allocator.hpp:179-183 (default size 8 MiB) */
        explicit Allocator(int dev = 0, cudaStream_t queue = nullptr, size_t size = 8U * 1024U * 1024U)
            : device_(dev)
        {
            alloc(queue, size);
        }

        ~Allocator()
        {
            if(heap_ != nullptr)
                mmc_heap_destroy(heap_);
            else
                mmc_oldmalloc_set_heap(8192u, device_); /* CudaSetLimits::resetMemPool; fails after use, ignored */
        }

        /* allocator.hpp:195-200 */
        void destructiveResize(int /*dev*/, cudaStream_t queue, size_t size)
        {
            if(heap_ == nullptr)
            {
                detail::throw_status(mmc_oldmalloc_set_heap(size, device_), "destructiveResize");
                return;
            }
            detail::throw_status(mmc_heap_destructive_resize(heap_, size, queue), "destructiveResize");
            mmc_heap_device_handle(heap_, &handle_);
        }

        /* allocator.hpp:202-212 */
        auto getAllocatorHandle() const -> AllocatorHandle { return AllocatorHandle{handle_}; }
        operator AllocatorHandle() const { return getAllocatorHandle(); }

        /* allocator.hpp:214-223 */
        static auto info(std::string linebreak = " ") -> std::string
        {
            std::stringstream ss;
            ss << "CreationPolicy:      " << CreationPolicy::classname() << "    " << linebreak;
            ss << "DistributionPolicy:  " << DistributionPolicy::classname() << "" << linebreak;
            ss << "OOMPolicy:           " << OOMPolicy::classname() << "         " << linebreak;
            ss << "ReservePoolPolicy:   " << ReservePoolPolicy::classname() << " " << linebreak;
            ss << "AlignmentPolicy:     " << AlignmentPolicy::classname() << "   " << linebreak;
            return ss.str();
        }

        /* allocator.hpp:227-233: pads, counts, waits */
        auto getAvailableSlots(int /*dev*/, cudaStream_t queue, size_t slotSize) -> unsigned
        {
            if constexpr(!CreationPolicy::providesAvailableSlots)
                return 0u; /* allocator.hpp:47-55 */
            unsigned out = 0;
            detail::throw_status(mmc_available_slots(heap_, slotSize, queue, &out), "getAvailableSlots");
            return out;
        }

        /* allocator.hpp:235-241 (OldMalloc has no pool of its own: {nullptr, 0}) */
        auto getHeapLocations() -> HeapInfoVector
        {
            HeapInfo hi{};
            if(heap_ != nullptr)
                mmc_heap_locations(heap_, &hi.p, &hi.size);
            return HeapInfoVector{hi};
        }

        /* device error bits (MMC_DEVERR_*), e.g. from BadAllocException */
        auto errorFlags(cudaStream_t queue = nullptr, bool clear = false) -> uint32_t
        {
            uint32_t f = 0;
            if(heap_ != nullptr)
                detail::throw_status(mmc_heap_error(heap_, queue, &f, clear ? 1 : 0), "errorFlags");
            return f;
        }

        auto cHeap() const -> mmc_heap* { return heap_; }

    private:
        void alloc(cudaStream_t queue, size_t size)
        {
            if constexpr(!CreationPolicy::usesHeap)
            {
                /* CudaSetLimits::setMemPool (CudaSetLimits.hpp:59-64); OldMalloc's
                 * initHeap does nothing (OldMalloc.hpp:73-81) */
                detail::throw_status(mmc_oldmalloc_set_heap(size, device_), "Allocator");
                return;
            }
            mmc_config c;
            mmc_config_default(&c);
            CreationPolicy::fill(c);
            c.distribution = DistributionPolicy::code;
            c.oom_policy = OOMPolicy::code;
            c.dataAlignment = static_cast<uint32_t>(AlignmentPolicy::dataAlignment);
            detail::throw_status(mmc_heap_create(&c, size, device_, queue, &heap_), "Allocator");
            mmc_heap_device_handle(heap_, &handle_);
        }

        int device_;
        mmc_heap* heap_ = nullptr;
        mmc_device_handle handle_{};
    };

    /* mallocMC_traits.hpp:33-37 */
    template<class T_Allocator>
    struct Traits
    {
        static constexpr bool providesAvailableSlots = T_Allocator::CreationPolicy::providesAvailableSlots;
    };
} // namespace mallocMC

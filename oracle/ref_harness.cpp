/* Reference harness: drives the UNMODIFIED reference mallocMC headers
 * (src/include/mallocMC, alpaka 1.0.0 CPU-serial backend) through a small
 * op program and prints every result as one JSON document.
 *
 * TEST INFRASTRUCTURE ONLY. Built by oracle/Makefile into oracle/_ref/ from the
 * reference sources where they lie; used to generate tests/golden fixtures
 * that pin the C restatement (oracle/scatter_oracle.c). Nothing in the product
 * path links or runs this.
 *
 * Program format (one op per line, read from stdin):
 *   m <bytes>     handle.malloc in a 1x1 kernel   -> pool offset or -1
 *   f <k>         handle.free(pointer returned by the k-th "m")
 *   s <bytes>     Allocator::getAvailableSlots (host; 64 blocks on CPU-serial)
 *   d <bytes>     handle.getAvailableSlots in a 1x1 kernel (accelerator path)
 *   snap          metadata snapshot (sparse PTEs, regions, on-page mask words)
 * The heap size and configuration come from argv: <config-name> <heap-bytes>.
 */

#include <alpaka/alpaka.hpp>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

/* Compile prelude (no reference file is edited):
 * 1. mallocMC_utils.hpp names alpaka::AccGpuUniformCudaHipRt, which alpaka only
 *    declares when a GPU backend is enabled; declare it for the CPU-only build.
 * 2. Scatter::calcAdditionalChunks calls alpaka::math::max/min with (int,
 *    unsigned). std::max cannot deduce that; CUDA's ::max/::min(int, unsigned)
 *    compare as unsigned, so these specialisations do the same. */
namespace alpaka
{
    template<typename TApi, typename TDim, typename TIdx>
    class AccGpuUniformCudaHipRt;

    namespace math::trait
    {
        template<>
        struct Max<MaxStdLib, int, unsigned, void>
        {
            auto operator()(MaxStdLib const&, int const& x, unsigned const& y) -> unsigned
            {
                return std::max(static_cast<unsigned>(x), y);
            }
        };
        template<>
        struct Min<MinStdLib, int, unsigned, void>
        {
            auto operator()(MinStdLib const&, int const& x, unsigned const& y) -> unsigned
            {
                return std::min(static_cast<unsigned>(x), y);
            }
        };
    } // namespace math::trait
} // namespace alpaka

#define ANALYSEHEAP 1 /* makes the Scatter metadata members public for the snapshot */
#include <mallocMC/mallocMC.hpp>

using Dim = alpaka::DimInt<1>;
using Idx = std::size_t;
using Acc = alpaka::AccCpuSerial<Dim, Idx>;
using Queue = alpaka::Queue<Acc, alpaka::Blocking>;

template<unsigned P, size_t AB, unsigned R, unsigned W, bool RESET>
struct HeapCfg
{
    static constexpr auto pagesize = P;
    static constexpr auto accessblocksize = AB;
    static constexpr auto regionsize = R;
    static constexpr auto wastefactor = W;
    static constexpr auto resetfreedpages = RESET;
};

template<unsigned K, unsigned MP, unsigned WP, unsigned WPREL>
struct HashCfg
{
    static constexpr auto hashingK = K;
    static constexpr auto hashingDistMP = MP;
    static constexpr auto hashingDistWP = WP;
    static constexpr auto hashingDistWPRel = WPREL;
};

template<unsigned P>
struct XCfg
{
    static constexpr auto pagesize = P;
};

template<unsigned A>
struct ShrinkCfg
{
    static constexpr auto dataAlignment = A;
};

using DefaultHash = HashCfg<38183, 17497, 1, 1>;

template<typename Scatter, typename Dist, typename Align>
using AllocT = mallocMC::Allocator<
    Acc,
    Scatter,
    Dist,
    mallocMC::OOMPolicies::ReturnNull,
    mallocMC::ReservePoolPolicies::AlpakaBuf<Acc>,
    Align>;

struct Op
{
    char kind;
    unsigned long long arg;
};

template<typename Alloc>
int run(const char* name, size_t heapBytes, std::vector<Op> const& prog)
{
    using Handle = typename Alloc::AllocatorHandle;
    using Creation = typename Alloc::CreationPolicy;
    auto const platform = alpaka::Platform<Acc>{};
    auto const dev = alpaka::getDevByIdx(platform, 0);
    auto queue = Queue{dev};
    Alloc alloc(dev, queue, heapBytes);
    Handle h = alloc.getAllocatorHandle();
    auto* devAlloc = h.devAllocator;
    char* pool = static_cast<char*>(alloc.getHeapLocations()[0].p);

    std::vector<void*> ptrs;
    std::ostringstream out;
    out << "{\"config\":\"" << name << "\",\"heap_bytes\":" << heapBytes
        << ",\"pool_misalign\":" << (reinterpret_cast<uintptr_t>(pool) & 15u)
        << ",\"numpages\":" << devAlloc->_numpages << ",\"accessblocks\":" << devAlloc->_accessblocks
        << ",\"pages_offset_from_pool\":" << (reinterpret_cast<char*>(devAlloc->_page) - pool)
        << ",\"ptes_offset_from_pool\":" << (reinterpret_cast<char const volatile*>(devAlloc->_ptes) - pool)
        << ",\"regions_offset_from_pool\":" << (reinterpret_cast<char const volatile*>(devAlloc->_regions) - pool)
        << ",\"results\":[";
    bool first = true;
    auto const wd1 = alpaka::WorkDivMembers<Dim, Idx>{Idx{1}, Idx{1}, Idx{1}};
    std::vector<std::string> snaps;

    for(auto const& op : prog)
    {
        std::ostringstream r;
        if(op.kind == 'm')
        {
            void* result = nullptr;
            auto k = [] ALPAKA_FN_ACC(Acc const& acc, Handle hh, size_t n, void** res) { *res = hh.malloc(acc, n); };
            alpaka::enqueue(queue, alpaka::createTaskKernel<Acc>(wd1, k, h, static_cast<size_t>(op.arg), &result));
            alpaka::wait(queue);
            ptrs.push_back(result);
            long long off = result ? static_cast<long long>(static_cast<char*>(result) - pool) : -1;
            r << "[\"m\"," << op.arg << "," << off << "]";
        }
        else if(op.kind == 'f')
        {
            void* p = ptrs.at(op.arg);
            auto k = [] ALPAKA_FN_ACC(Acc const& acc, Handle hh, void* q) { hh.free(acc, q); };
            alpaka::enqueue(queue, alpaka::createTaskKernel<Acc>(wd1, k, h, p));
            alpaka::wait(queue);
            r << "[\"f\"," << op.arg << "]";
        }
        else if(op.kind == 's')
        {
            unsigned v = alloc.getAvailableSlots(dev, queue, static_cast<size_t>(op.arg));
            r << "[\"s\"," << op.arg << "," << v << "]";
        }
        else if(op.kind == 'd')
        {
            unsigned v = 0;
            auto k = [] ALPAKA_FN_ACC(Acc const& acc, Handle hh, size_t n, unsigned* res)
            { *res = hh.getAvailableSlots(acc, n); };
            alpaka::enqueue(queue, alpaka::createTaskKernel<Acc>(wd1, k, h, static_cast<size_t>(op.arg), &v));
            alpaka::wait(queue);
            r << "[\"d\"," << op.arg << "," << v << "]";
        }
        else if(op.kind == 'S')
        {
            /* metadata snapshot: sparse non-zero PTEs, region counters, on-page
             * mask words (the last maxOnPageMasks words of each page), header */
            constexpr unsigned P = Creation::_pagesize;
            constexpr unsigned nmask = Creation::maxOnPageMasks;
            std::ostringstream s;
            s << "{\"ptes\":[";
            bool f1 = true;
            for(unsigned i = 0; i < devAlloc->_numpages; ++i)
            {
                auto const& e = devAlloc->_ptes[i];
                if(e.chunksize || e.count || e.bitmask)
                {
                    s << (f1 ? "" : ",") << "[" << i << "," << e.chunksize << "," << e.count << "," << e.bitmask
                      << "]";
                    f1 = false;
                }
            }
            s << "],\"regions\":[";
            f1 = true;
            unsigned const numregions = devAlloc->_numpages / Creation::_regionsize;
            for(unsigned i = 0; i < numregions; ++i)
                if(devAlloc->_regions[i])
                {
                    s << (f1 ? "" : ",") << "[" << i << "," << devAlloc->_regions[i] << "]";
                    f1 = false;
                }
            s << "],\"masks\":[";
            f1 = true;
            for(unsigned i = 0; i < devAlloc->_numpages; ++i)
            {
                auto const* w = reinterpret_cast<std::uint32_t const*>(devAlloc->_page[i].data + P - 4 * nmask);
                for(unsigned j = 0; j < nmask; ++j)
                    if(w[j])
                    {
                        /* index counted from the end of the page: 1 = last word */
                        s << (f1 ? "" : ",") << "[" << i << "," << (nmask - j) << "," << w[j] << "]";
                        f1 = false;
                    }
            }
            s << "],\"firstFreePageBased\":" << devAlloc->_firstFreePageBased
              << ",\"firstfreeblock\":" << devAlloc->_firstfreeblock
              << ",\"pagebasedMutex\":" << devAlloc->_pagebasedMutex << "}";
            snaps.push_back(s.str());
            r << "[\"snap\"," << (snaps.size() - 1) << "]";
        }
        out << (first ? "" : ",") << r.str();
        first = false;
    }
    out << "],\"snapshots\":[";
    for(size_t i = 0; i < snaps.size(); ++i)
        out << (i ? "," : "") << snaps[i];
    out << "]}";
    std::cout << out.str() << std::endl;
    return 0;
}

/* The configuration table. Names are stable: tests/golden fixtures refer to them. */
namespace MC = mallocMC;
using p4k_ab8m_r16_w2 = AllocT<
    MC::CreationPolicies::Scatter<HeapCfg<4096, 8u << 20, 16, 2, false>, DefaultHash>,
    MC::DistributionPolicies::XMallocSIMD<XCfg<4096>>,
    MC::AlignmentPolicies::Shrink<ShrinkCfg<16>>>;
using p4k_ab8m_r16_w2_reset = AllocT<
    MC::CreationPolicies::Scatter<HeapCfg<4096, 8u << 20, 16, 2, true>, DefaultHash>,
    MC::DistributionPolicies::XMallocSIMD<XCfg<4096>>,
    MC::AlignmentPolicies::Shrink<ShrinkCfg<16>>>;
using p4k_ab4m_r8_w4_noop = AllocT<
    MC::CreationPolicies::Scatter<HeapCfg<4096, 4u << 20, 8, 4, false>, HashCfg<7919, 101, 3, 2>>,
    MC::DistributionPolicies::Noop,
    MC::AlignmentPolicies::Noop>;
using p16k_ab16m_r8_w2 = AllocT<
    MC::CreationPolicies::Scatter<HeapCfg<16384, 16u << 20, 8, 2, false>, DefaultHash>,
    MC::DistributionPolicies::XMallocSIMD<XCfg<16384>>,
    MC::AlignmentPolicies::Shrink<ShrinkCfg<16>>>;
using p64k_ab32m_r4_w2_reset = AllocT<
    MC::CreationPolicies::Scatter<HeapCfg<65536, 32u << 20, 4, 2, true>, DefaultHash>,
    MC::DistributionPolicies::XMallocSIMD<XCfg<65536>>,
    MC::AlignmentPolicies::Shrink<ShrinkCfg<16>>>;
using p1k_ab1m_r32_w1_a8 = AllocT<
    MC::CreationPolicies::Scatter<HeapCfg<1024, 1u << 20, 32, 1, false>, DefaultHash>,
    MC::DistributionPolicies::XMallocSIMD<XCfg<1024>>,
    MC::AlignmentPolicies::Shrink<ShrinkCfg<8>>>;

#define CFG_LIST(X)                                                                                                   \
    X(p4k_ab8m_r16_w2)                                                                                                \
    X(p4k_ab8m_r16_w2_reset)                                                                                          \
    X(p4k_ab4m_r8_w4_noop)                                                                                            \
    X(p16k_ab16m_r8_w2)                                                                                               \
    X(p64k_ab32m_r4_w2_reset)                                                                                         \
    X(p1k_ab1m_r32_w1_a8)

int main(int argc, char** argv)
{
    if(argc < 3)
    {
        std::cerr << "usage: " << argv[0] << " <config> <heap-bytes> < program\n";
        return 2;
    }
    std::string const name = argv[1];
    size_t const heapBytes = std::stoull(argv[2]);
    std::vector<Op> prog;
    std::string tok;
    while(std::cin >> tok)
    {
        if(tok == "snap")
            prog.push_back({'S', 0});
        else
        {
            unsigned long long a = 0;
            std::cin >> a;
            prog.push_back({tok[0], a});
        }
    }
#define X(n)                                                                                                          \
    if(name == #n)                                                                                                    \
        return run<n>(#n, heapBytes, prog);
    CFG_LIST(X)
#undef X
    std::cerr << "unknown config " << name << "\n";
    return 2;
}

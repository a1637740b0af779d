/* Reference CPU baseline: the full-GPU uniform stress run by the UNMODIFIED
 * reference mallocMC headers on one of alpaka 1.0.0's CPU backends, timed on
 * the host cores.
 *
 * TEST AND BENCHMARK INFRASTRUCTURE ONLY. Built by oracle/Makefile into
 * oracle/_ref/ from the reference sources (ref_prelude.h force-included, the
 * Boost stand-in of shim/), twice:
 *   ref_stress_omp     alpaka::AccCpuOmp2Blocks (-fopenmp): the grid's blocks
 *                      run on OMP_NUM_THREADS host threads, one thread per
 *                      block (alpaka/include/alpaka/acc/AccCpuOmp2Blocks.hpp);
 *   ref_stress_serial  alpaka::AccCpuSerial, one host thread
 *                      (alpaka/include/alpaka/acc/AccCpuSerial.hpp:140-141).
 * bench.py times it as the reference arm and as the line's cpu_baseline. The
 * product path never links or runs it.
 *
 * Workload (what the GPU stress kernel does per thread, mallocmc_gb300/csrc/
 * workloads.cu): every virtual thread t runs `rounds` iterations r of
 *   m = mix64(seed, t, r); size = lo + ((m >> 32) % nsizes) * step;
 *   p = handle.malloc(acc, size); write the u64 pattern m + i over the block;
 *   read it back and count mismatches; handle.free(acc, p).
 * A virtual thread is one alpaka block of one thread (the CPU backends'
 * shape), as the reference's own tests run GPU grids on the CPU.
 *
 * Usage: ref_stress <config> <heap-bytes> <threads> <rounds> <seed> <warmup>
 *                   <steps> <target-seconds>
 *   threads: the full workload's thread count; a step runs min(threads, a
 *   calibrated count that takes about target-seconds) virtual threads, with
 *   seed + step as its seed. Prints one JSON line per timed step and a summary.
 */
#include <alpaka/alpaka.hpp>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#ifdef _OPENMP
#    include <omp.h>
#endif

#include <mallocMC/mallocMC.hpp>

using Dim = alpaka::DimInt<1>;
using Idx = std::size_t;
#if defined(ALPAKA_ACC_CPU_B_OMP2_T_SEQ_ENABLED)
using Acc = alpaka::AccCpuOmp2Blocks<Dim, Idx>;
static char const* const kBackend = "alpaka AccCpuOmp2Blocks";
#else
using Acc = alpaka::AccCpuSerial<Dim, Idx>;
static char const* const kBackend = "alpaka AccCpuSerial";
#endif
using Queue = alpaka::Queue<Acc, alpaka::Blocking>;

namespace
{
    template<unsigned P, size_t AB, unsigned R, unsigned W>
    struct HeapCfg
    {
        static constexpr auto pagesize = P;
        static constexpr auto accessblocksize = AB;
        static constexpr auto regionsize = R;
        static constexpr auto wastefactor = W;
        static constexpr auto resetfreedpages = false;
    };

    /* the reference's DefaultScatterHashingParams (Scatter.hpp:77-85) */
    struct Hash
    {
        static constexpr auto hashingK = 38183u;
        static constexpr auto hashingDistMP = 17497u;
        static constexpr auto hashingDistWP = 1u;
        static constexpr auto hashingDistWPRel = 1u;
    };

    struct XCfg
    {
        static constexpr auto pagesize = 4096u;
    };

    struct ShrinkCfg
    {
        static constexpr auto dataAlignment = 16u;
    };

    template<size_t AB>
    using AllocT = mallocMC::Allocator<
        Acc,
        mallocMC::CreationPolicies::Scatter<HeapCfg<4096, AB, 16, 2>, Hash>,
        mallocMC::DistributionPolicies::XMallocSIMD<XCfg>,
        mallocMC::OOMPolicies::ReturnNull,
        mallocMC::ReservePoolPolicies::AlpakaBuf<Acc>,
        mallocMC::AlignmentPolicies::Shrink<ShrinkCfg>>;

    /* SplitMix64-style counter hash, the same function the GPU kernels draw with */
    ALPAKA_FN_HOST_ACC inline std::uint64_t mix64(std::uint64_t seed, std::uint64_t a, std::uint64_t b)
    {
        std::uint64_t z = seed + a * 0x9E3779B97F4A7C15ull + b * 0xD1B54A32D192ED03ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }

    struct StressParams
    {
        std::uint32_t rounds, lo, hi, step;
        std::uint64_t seed;
    };

    /* One virtual thread per block; per-thread results, summed on the host. */
    struct StressKernel
    {
        template<typename TAcc, typename Handle>
        ALPAKA_FN_ACC void operator()(
            TAcc const& acc,
            Handle h,
            StressParams p,
            std::uint64_t* pairs,
            std::uint64_t* nulls,
            std::uint64_t* bad) const
        {
            auto const t = alpaka::getIdx<alpaka::Grid, alpaka::Threads>(acc)[0];
            std::uint32_t const nsizes = (p.hi - p.lo) / p.step + 1u;
            std::uint64_t np = 0, nn = 0, nb = 0;
            for(std::uint32_t r = 0; r < p.rounds; ++r)
            {
                std::uint64_t const m = mix64(p.seed, t, r);
                std::uint32_t const bytes = p.lo + static_cast<std::uint32_t>((m >> 32) % nsizes) * p.step;
                auto* q = static_cast<std::uint64_t*>(h.malloc(acc, bytes));
                if(q == nullptr)
                {
                    ++nn;
                    continue;
                }
                std::uint32_t const n8 = bytes / 8u;
                for(std::uint32_t i = 0; i < n8; ++i)
                    q[i] = m + i;
                for(std::uint32_t i = 0; i < n8; ++i)
                    nb += q[i] != m + i;
                h.free(acc, q);
                ++np;
            }
            pairs[t] = np;
            nulls[t] = nn;
            bad[t] = nb;
        }
    };

    struct StepResult
    {
        std::uint64_t pairs = 0, nulls = 0, bad = 0;
        double seconds = 0.0;
    };

    template<typename Alloc>
    int run(char const* name, size_t heapBytes, size_t threads, std::uint32_t rounds, std::uint64_t seed, int warmup,
            int steps, double target)
    {
        auto const platform = alpaka::Platform<Acc>{};
        auto const dev = alpaka::getDevByIdx(platform, 0);
        auto queue = Queue{dev};
        auto const t0 = std::chrono::steady_clock::now();
        Alloc alloc(dev, queue, heapBytes);
        auto const t1 = std::chrono::steady_clock::now();
        auto h = alloc.getAllocatorHandle();
        int workers = 1;
#ifdef _OPENMP
        workers = omp_get_max_threads();
#endif
        std::vector<std::uint64_t> pairs(threads), nulls(threads), bad(threads);

        auto step = [&](size_t n, std::uint32_t rr, std::uint64_t sd) -> StepResult
        {
            StressParams p{rr, 16u, 1024u, 16u, sd};
            auto const wd = alpaka::WorkDivMembers<Dim, Idx>{Idx{n}, Idx{1}, Idx{1}};
            auto const a = std::chrono::steady_clock::now();
            alpaka::enqueue(
                queue,
                alpaka::createTaskKernel<Acc>(wd, StressKernel{}, h, p, pairs.data(), nulls.data(), bad.data()));
            alpaka::wait(queue);
            auto const b = std::chrono::steady_clock::now();
            StepResult s;
            s.seconds = std::chrono::duration<double>(b - a).count();
            for(size_t i = 0; i < n; ++i)
            {
                s.pairs += pairs[i];
                s.nulls += nulls[i];
                s.bad += bad[i];
            }
            return s;
        };

        /* calibrate: virtual threads per step for about `target` seconds */
        size_t const cal_n = std::min<size_t>(threads, static_cast<size_t>(workers) * 256u);
        StepResult const cal = step(cal_n, 4u, seed ^ 0xCA11B8A7Eull);
        double const rate = cal.seconds > 0.0 ? static_cast<double>(cal.pairs) / cal.seconds : 1e6;
        size_t n = static_cast<size_t>(target * rate / rounds);
        n = std::max<size_t>(n, std::min<size_t>(threads, 1024u));
        n = std::min(n, threads);

        StepResult total;
        for(int i = 0; i < warmup + steps; ++i)
        {
            StepResult const s = step(n, rounds, seed + 1u + static_cast<std::uint64_t>(i));
            if(i < warmup)
                continue;
            std::printf(
                "{\"step\": %d, \"pairs\": %llu, \"nulls\": %llu, \"bad\": %llu, \"seconds\": %.6f}\n",
                i - warmup,
                static_cast<unsigned long long>(s.pairs),
                static_cast<unsigned long long>(s.nulls),
                static_cast<unsigned long long>(s.bad),
                s.seconds);
            total.pairs += s.pairs;
            total.nulls += s.nulls;
            total.bad += s.bad;
            total.seconds += s.seconds;
        }
        std::printf(
            "{\"summary\": true, \"backend\": \"%s\", \"config\": \"%s\", \"heap_bytes\": %zu, \"workers\": %d, "
            "\"virtual_threads\": %zu, \"rounds\": %u, \"steps\": %d, \"pairs\": %llu, \"nulls\": %llu, "
            "\"bad\": %llu, \"seconds\": %.6f, \"heap_init_seconds\": %.3f}\n",
            kBackend,
            name,
            heapBytes,
            workers,
            n,
            rounds,
            steps,
            static_cast<unsigned long long>(total.pairs),
            static_cast<unsigned long long>(total.nulls),
            static_cast<unsigned long long>(total.bad),
            total.seconds,
            std::chrono::duration<double>(t1 - t0).count());
        std::fflush(stdout);
        return 0;
    }
} // namespace

/* Heap configurations: pagesize 4096, regionsize 16, wastefactor 2, no page
 * reset, the reference's hash, XMallocSIMD<4096>, ReturnNull, Shrink<16>; the
 * access block is 4 GiB (the bench's default), 2 GiB (the reference's) or
 * 8 MiB (small heaps for tests). */
using p4k_ab4g_r16_w2 = AllocT<size_t{4096} << 20>;
using p4k_ab2g_r16_w2 = AllocT<size_t{2048} << 20>;
using p4k_ab8m_r16_w2 = AllocT<size_t{8} << 20>;

int main(int argc, char** argv)
{
    if(argc < 9)
    {
        std::fprintf(
            stderr,
            "usage: %s <config> <heap-bytes> <threads> <rounds> <seed> <warmup> <steps> <target-seconds>\n",
            argv[0]);
        return 2;
    }
    std::string const name = argv[1];
    size_t const heap = std::stoull(argv[2]);
    size_t const threads = std::stoull(argv[3]);
    auto const rounds = static_cast<std::uint32_t>(std::stoul(argv[4]));
    auto const seed = static_cast<std::uint64_t>(std::stoull(argv[5]));
    int const warmup = std::stoi(argv[6]);
    int const steps = std::stoi(argv[7]);
    double const target = std::stod(argv[8]);
    if(name == "p4k_ab4g_r16_w2")
        return run<p4k_ab4g_r16_w2>(name.c_str(), heap, threads, rounds, seed, warmup, steps, target);
    if(name == "p4k_ab2g_r16_w2")
        return run<p4k_ab2g_r16_w2>(name.c_str(), heap, threads, rounds, seed, warmup, steps, target);
    if(name == "p4k_ab8m_r16_w2")
        return run<p4k_ab8m_r16_w2>(name.c_str(), heap, threads, rounds, seed, warmup, steps, target);
    std::fprintf(stderr, "unknown config %s\n", name.c_str());
    return 2;
}

/* verify_heap — the reference's heap verification tool (tests/verify_heap.cpp
 * with tests/verify_heap_config.hpp), written against the C++ drop-in API.
 *
 * Every thread allocates slots of 750 x u64 (6000 bytes: the multi-page path
 * with 4 KiB pages) until the heap returns NULL, fills each with its global
 * index (offset + i); the device then verifies every element and the content
 * sum, one element is damaged and the verification must now fail (the
 * negative check), and everything is freed. Same command line
 * (verify_heap.cpp:122-182) and, with -m, the same CSV header and values
 * (verify_heap.cpp:531-603, including its "Wastefactor" column that carries
 * the wasted bytes). Exit status 0 when the verification is correct.
 *
 * The allocator is the reference's (Scatter 4096 / 2 GiB / 16 / 2 / no reset,
 * Noop distribution, ReturnNull, Shrink 16). A heap below 2 GiB holds no whole
 * access block of that size (the page area is about 0.3 % smaller than the
 * heap); the reference then divides by zero (Scatter.hpp:991-993) and this
 * library refuses the configuration, so such heaps run the same allocator with
 * a 256 MiB access block (8 MiB when even that does not fit), which -v reports.
 *
 * --blocks and --threads mean what the reference's help text says; the
 * reference's main() passes them to run_heap_verification in swapped order
 * (verify_heap.cpp:95 against :619), so its CSV shows --threads as Gridsize.
 *
 * Additions: the content sum is also checked against the Gaussian sum of
 * 0 .. usedSlots*750-1 (the check the reference's comments describe,
 * verify_heap.cpp:495-498), and the heap's device error flags must be clear.
 */
#include "mallocMC/mallocMC.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <sstream>
#include <string>

namespace
{
    constexpr unsigned ELEMS_PER_SLOT = 750;
    using allocElem_t = unsigned long long;
    using Acc = mallocMC::AccGpuCuda;

    template<unsigned T_AccessBlock>
    struct ScatterConfig
    {
        static constexpr auto pagesize = 4096;
        static constexpr auto accessblocksize = T_AccessBlock;
        static constexpr auto regionsize = 16;
        static constexpr auto wastefactor = 2;
        static constexpr auto resetfreedpages = false;
    };
    struct ScatterHashParams
    {
        static constexpr auto hashingK = 38183;
        static constexpr auto hashingDistMP = 17497;
        static constexpr auto hashingDistWP = 1;
        static constexpr auto hashingDistWPRel = 1;
    };
    struct AlignmentConfig
    {
        static constexpr auto dataAlignment = 16;
    };
    template<unsigned T_AccessBlock>
    using ScatterAllocator = mallocMC::Allocator<
        Acc,
        mallocMC::CreationPolicies::Scatter<ScatterConfig<T_AccessBlock>, ScatterHashParams>,
        mallocMC::DistributionPolicies::Noop,
        mallocMC::OOMPolicies::ReturnNull,
        mallocMC::ReservePoolPolicies::AlpakaBuf<Acc>,
        mallocMC::AlignmentPolicies::Shrink<AlignmentConfig>>;

    bool verbose = false;

    std::ostream& dout()
    {
        static std::ostream null_stream(nullptr);
        return verbose ? std::cout : null_stream;
    }

    /* AllocAll (verify_heap.cpp:333-361); `capacity` bounds the pointer array */
    template<class Handle>
    __global__ void allocAll(allocElem_t** data, unsigned long long* counter, unsigned long long* globalSum,
                             unsigned long long capacity, Handle mMC)
    {
        const Acc acc{};
        unsigned long long sum = 0;
        while(true)
        {
            allocElem_t* p = static_cast<allocElem_t*>(mMC.malloc(acc, sizeof(allocElem_t) * ELEMS_PER_SLOT));
            if(p == nullptr)
                break;
            const unsigned long long pos = atomicAdd(counter, 1ull);
            if(pos >= capacity)
            {
                mMC.free(acc, p);
                break;
            }
            const unsigned long long offset = pos * ELEMS_PER_SLOT;
            for(unsigned i = 0; i < ELEMS_PER_SLOT; ++i)
            {
                p[i] = static_cast<allocElem_t>(offset + i);
                sum += static_cast<unsigned long long>(p[i]);
            }
            data[pos] = p;
        }
        atomicAdd(globalSum, sum);
    }

    /* Check_content (verify_heap.cpp:241-274) */
    __global__ void checkContent(allocElem_t** data, unsigned long long* counter, unsigned long long* globalSum,
                                 unsigned long long nSlots, int* correct)
    {
        unsigned long long sum = 0;
        while(true)
        {
            const unsigned long long pos = atomicAdd(counter, 1ull);
            if(pos >= nSlots)
                break;
            const unsigned long long offset = pos * ELEMS_PER_SLOT;
            for(unsigned i = 0; i < ELEMS_PER_SLOT; ++i)
            {
                if(static_cast<allocElem_t>(data[pos][i]) != static_cast<allocElem_t>(offset + i))
                    atomicAnd(correct, 0);
                sum += static_cast<unsigned long long>(data[pos][i]);
            }
        }
        atomicAdd(globalSum, sum);
    }

    /* DeallocAll (verify_heap.cpp:371-388) */
    template<class Handle>
    __global__ void deallocAll(allocElem_t** data, unsigned long long* counter, unsigned long long nSlots, Handle mMC)
    {
        const Acc acc{};
        while(true)
        {
            const unsigned long long pos = atomicAdd(counter, 1ull);
            if(pos >= nSlots)
                break;
            mMC.free(acc, data[pos]);
        }
    }

    /* DamageElement (verify_heap.cpp:399-405) */
    __global__ void damageElement(allocElem_t** data)
    {
        data[1][0] = static_cast<allocElem_t>(5 * ELEMS_PER_SLOT - 1);
    }

    bool cuda_ok(cudaError_t e, const char* what)
    {
        if(e == cudaSuccess)
            return true;
        std::cerr << what << ": " << cudaGetErrorString(e) << "\n";
        return false;
    }

    /* verify (verify_heap.cpp:479-523): content check on the device, plus the sum */
    bool verify(allocElem_t** d_data, unsigned long long nSlots, unsigned blocks, unsigned threads,
                unsigned long long* sum_out)
    {
        dout() << "verifying on device... ";
        unsigned long long* d_buf = nullptr; /* [sum, counter, correct] */
        if(!cuda_ok(cudaMalloc(&d_buf, 3 * sizeof(unsigned long long)), "cudaMalloc"))
            return false;
        const unsigned long long init[3] = {0ull, 0ull, 1ull};
        cudaMemcpy(d_buf, init, sizeof(init), cudaMemcpyHostToDevice);
        checkContent<<<blocks, threads>>>(d_data, d_buf + 1, d_buf, nSlots, reinterpret_cast<int*>(d_buf + 2));
        unsigned long long out[3] = {0ull, 0ull, 0ull};
        const bool ok = cuda_ok(cudaMemcpy(out, d_buf, sizeof(out), cudaMemcpyDeviceToHost), "verify");
        cudaFree(d_buf);
        const bool correct = ok && (out[2] & 0xFFFFFFFFull) != 0ull;
        *sum_out = out[0];
        dout() << (correct ? "done\n" : "failed\n");
        return correct;
    }

    /* sum of 0 .. n-1 modulo 2^64 (the device sums wrap the same way) */
    unsigned long long gauss(unsigned long long n)
    {
        if(n == 0)
            return 0;
        return (n % 2 == 0) ? (n / 2) * (n - 1) : n * ((n - 1) / 2);
    }

    /* print_machine_readable (verify_heap.cpp:531-603): same columns, same values */
    void print_machine_readable(unsigned pagesize, unsigned accessblocks, unsigned regionsize, bool resetfreedpages,
                                unsigned blocks, unsigned threads, unsigned elemsPerSlot, size_t allocElemSize,
                                size_t heapSize, size_t maxSpace, size_t maxSlots, unsigned long long usedSlots,
                                float allocFrac, size_t wasted, bool correct)
    {
        const char* sep = ",";
        std::stringstream h, v;
        h << "PagesizeByte" << sep << "Accessblocks" << sep << "Regionsize" << sep << "Wastefactor" << sep
          << "ResetFreedPage" << sep << "Gridsize" << sep << "Blocksize" << sep << "ELEMS_PER_SLOT" << sep
          << "allocElemByte" << sep << "heapsizeByte" << sep << "maxSpaceByte" << sep << "maxSlots" << sep
          << "usedSlots" << sep << "allocFraction" << sep << "wastedBytes" << sep << "correct";
        v << pagesize << sep << accessblocks << sep << regionsize << sep << wasted << sep << resetfreedpages << sep
          << blocks << sep << threads << sep << elemsPerSlot << sep << allocElemSize << sep << heapSize << sep
          << maxSpace << sep << maxSlots << sep << usedSlots << sep << allocFrac << sep << wasted << sep << correct;
        std::cout << h.str() << '\n' << v.str() << '\n';
    }

    /* run_heap_verification (verify_heap.cpp:617-738) */
    template<unsigned T_AccessBlock>
    bool run_heap_verification(int device, size_t heapMB, unsigned blocks, unsigned threads, bool machine_readable)
    {
        using Alloc = ScatterAllocator<T_AccessBlock>;
        using Cfg = ScatterConfig<T_AccessBlock>;
        cudaDeviceProp prop{};
        cudaGetDeviceProperties(&prop, device);
        threads = std::min(threads, static_cast<unsigned>(prop.maxThreadsPerBlock));

        const size_t heapSize = size_t(1024U * 1024U) * heapMB;
        const size_t slotSize = sizeof(allocElem_t) * ELEMS_PER_SLOT;
        const size_t nPointers = (heapSize + slotSize - 1) / slotSize;
        const size_t maxSlots = heapSize / slotSize;
        const size_t maxSpace = maxSlots * slotSize + nPointers * sizeof(allocElem_t*);
        bool correct = true;

        dout() << "CreationPolicy Arguments:\n"
               << "Pagesize:              " << Cfg::pagesize << '\n'
               << "Accessblocksize        " << Cfg::accessblocksize << '\n'
               << "Regionsize:            " << Cfg::regionsize << '\n'
               << "Wastefactor:           " << Cfg::wastefactor << '\n'
               << "ResetFreedPages        " << Cfg::resetfreedpages << "\n\n"
               << "Gridsize:              " << blocks << '\n'
               << "Blocksize:             " << threads << '\n'
               << "Allocated elements:    " << ELEMS_PER_SLOT << " x " << sizeof(allocElem_t) << "    Byte ("
               << slotSize << " Byte)\n"
               << "Heap:                  " << heapSize << " Byte (" << heapSize / std::pow(1024, 2) << " MByte)\n"
               << "max space w/ pointers: " << maxSpace << " Byte (" << maxSpace / std::pow(1024, 2) << " MByte)\n"
               << "maximum of elements:   " << maxSlots << '\n';

        unsigned long long usedSlots = 0, sumAllocElems = 0;
        float allocFrac = 0;
        size_t wasted = 0;
        {
            Alloc mMC(device, nullptr, heapSize);
            allocElem_t** d_data = nullptr;
            unsigned long long* d_cnt = nullptr; /* [nSlots, sum, dealloc counter] */
            if(!cuda_ok(cudaMalloc(&d_data, sizeof(allocElem_t*) * std::max<size_t>(nPointers, 1)), "cudaMalloc")
               || !cuda_ok(cudaMalloc(&d_cnt, 3 * sizeof(unsigned long long)), "cudaMalloc"))
                return false;
            cudaMemset(d_cnt, 0, 3 * sizeof(unsigned long long));

            dout() << "allocating on device...";
            allocAll<<<blocks, threads>>>(d_data, d_cnt, d_cnt + 1, nPointers, mMC.getAllocatorHandle());
            unsigned long long h_cnt[2] = {0ull, 0ull};
            correct = cuda_ok(cudaMemcpy(h_cnt, d_cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost), "allocate") && correct;
            usedSlots = std::min<unsigned long long>(h_cnt[0], nPointers);
            sumAllocElems = h_cnt[1];
            dout() << "done\n";

            allocFrac = static_cast<float>(usedSlots) * 100 / maxSlots;
            wasted = heapSize - static_cast<size_t>(usedSlots) * slotSize;
            dout() << "allocated elements:    " << usedSlots << " (" << allocFrac << "%)\n"
                   << "wasted heap space:     " << wasted << " Byte (" << wasted / std::pow(1024, 2) << " MByte)\n";

            unsigned long long checkSum = 0;
            correct = correct && verify(d_data, usedSlots, blocks, threads, &checkSum);
            correct = correct && checkSum == sumAllocElems && checkSum == gauss(usedSlots * ELEMS_PER_SLOT);

            dout() << "damaging of element... ";
            if(usedSlots > 1)
                damageElement<<<1, 1>>>(d_data);
            dout() << "done\n";
            /* this verification must fail: the damage was done before */
            unsigned long long damagedSum = 0;
            correct = correct && usedSlots > 1 && !verify(d_data, usedSlots, blocks, threads, &damagedSum);

            dout() << "deallocation...        ";
            deallocAll<<<blocks, threads>>>(d_data, d_cnt + 2, usedSlots, mMC.getAllocatorHandle());
            correct = cuda_ok(cudaDeviceSynchronize(), "deallocate") && correct;
            correct = correct && mMC.errorFlags() == 0u;
            cudaFree(d_data);
            cudaFree(d_cnt);
        }
        dout() << "done \n";

        if(machine_readable)
            print_machine_readable(Cfg::pagesize, Cfg::accessblocksize, Cfg::regionsize, Cfg::resetfreedpages, blocks,
                                   threads, ELEMS_PER_SLOT, sizeof(allocElem_t), heapSize, maxSpace, maxSlots,
                                   usedSlots, allocFrac, wasted, correct);
        return correct;
    }

    void print_help(const char* prog)
    {
        std::cout << "SYNOPSIS:\n"
                  << prog << " [OPTIONS]\n\nOPTIONS:\n"
                  << "  -h, --help\n    Print this help message and exit\n\n"
                  << "  -v, --verbose\n    Print information about parameters and progress\n\n"
                  << "  -m, --machine_readable\n    Print all relevant parameters as CSV. This will\n"
                  << "    suppress all other output unless explicitly\n    requested with --verbose or -v\n\n"
                  << "  --threads=N\n    Set the number of threads per block (default 128)\n\n"
                  << "  --blocks=N\n    Set the number of blocks in the grid (default 64)\n\n"
                  << "  --heapsize=N\n    Set the heapsize to N Megabyte (default 1024)\n\n"
                  << "  --device=N\n    CUDA device ordinal (default 0)\n";
    }
} // namespace

int main(int argc, char** argv)
{
    bool machine_readable = false;
    size_t heapMB = 1024;
    unsigned threads = 128, blocks = 64;
    int device = 0;
    /* tokens ARG=PARAM or ARG (verify_heap.cpp:122-182) */
    for(int i = 1; i < argc; ++i)
    {
        const std::string tok = argv[i];
        const size_t eq = tok.find('=');
        const std::string key = tok.substr(0, eq);
        const std::string val = eq == std::string::npos ? "" : tok.substr(eq + 1);
        if(key == "-v" || key == "--verbose")
            verbose = true;
        else if(key == "--threads")
            threads = static_cast<unsigned>(std::atoi(val.c_str()));
        else if(key == "--blocks")
            blocks = static_cast<unsigned>(std::atoi(val.c_str()));
        else if(key == "--heapsize")
            heapMB = static_cast<size_t>(std::atoll(val.c_str()));
        else if(key == "--device")
            device = std::atoi(val.c_str());
        else if(key == "-h" || key == "--help")
        {
            print_help(argv[0]);
            return 0;
        }
        else if(key == "-m" || key == "--machine_readable")
            machine_readable = true;
    }
    if(threads == 0 || blocks == 0 || heapMB == 0)
    {
        std::cerr << "threads, blocks and heapsize must be positive\n";
        return 2;
    }
    if(!cuda_ok(cudaSetDevice(device), "cudaSetDevice"))
        return 1;

    bool correct = false;
    try
    {
        /* the page area of a heap of B bytes: floor(B / (regionsize * (12 + pagesize) + 4)) regions of
         * regionsize pages (Scatter.hpp:976-980) */
        const size_t heapBytes = size_t(1024U * 1024U) * heapMB;
        const size_t pageArea = heapBytes / (16u * (12u + 4096u) + 4u) * 16u * 4096u;
        if(pageArea >= (size_t(2) << 30))
            correct = run_heap_verification<2u * 1024u * 1024u * 1024u>(device, heapMB, blocks, threads,
                                                                        machine_readable);
        else if(pageArea >= (size_t(256) << 20))
        {
            dout() << "heap below one 2 GiB access block: using 256 MiB access blocks\n";
            correct = run_heap_verification<256u * 1024u * 1024u>(device, heapMB, blocks, threads, machine_readable);
        }
        else
        {
            dout() << "heap below one 2 GiB access block: using 8 MiB access blocks\n";
            correct = run_heap_verification<8u * 1024u * 1024u>(device, heapMB, blocks, threads, machine_readable);
        }
    }
    catch(const std::exception& e)
    {
        std::cerr << "error: " << e.what() << "\n";
        correct = false;
    }

    if(!machine_readable || verbose)
    {
        if(correct)
        {
            std::cout << "\033[0;32mverification successful \xE2\x9C\x94\033[0m\n";
            return 0;
        }
        std::cerr << "\033[0;31mverification failed\033[0m\n";
        return 1;
    }
    return correct ? 0 : 1;
}

/* Internal helpers shared by the translation units of libmallocmc_gb300.so. */
#pragma once

#include "mallocmc_gb300.h"
#include "mallocMC/scatter_device.cuh"

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <string>

/* Run the statements in __VA_ARGS__ with `Ids` naming the thread-id type the
 * heap's kernels are launched with: GpuIdsDefault (the policy values fixed at
 * compile time) when the handle holds the default configuration, GpuIds (read
 * from the handle) otherwise. */
#define MMC_DISPATCH_IDS(handle, ...)                                                                                 \
    do                                                                                                                 \
    {                                                                                                                  \
        if(mmc::dev::GpuIdsDefault::matches(handle))                                                                   \
        {                                                                                                              \
            using Ids = mmc::dev::GpuIdsDefault;                                                                       \
            __VA_ARGS__;                                                                                               \
        }                                                                                                              \
        else                                                                                                           \
        {                                                                                                              \
            using Ids = mmc::dev::GpuIds;                                                                              \
            __VA_ARGS__;                                                                                               \
        }                                                                                                              \
    } while(0)

/* As MMC_DISPATCH_IDS, for a launch whose largest request (bytes, before
 * padding) the host knows: when it fits a page after padding, the default
 * configuration's instance is the one without the multi-page path
 * (mmc::dev::SmallRequests). */
#define MMC_DISPATCH_IDS_SIZED(handle, max_request, ...)                                                              \
    do                                                                                                                 \
    {                                                                                                                  \
        if(mmc::dev::GpuIdsDefault::matches(handle))                                                                   \
        {                                                                                                              \
            if(mmc::dev::apply_padding(16u, (max_request)) <= (handle).pagesize)                                      \
            {                                                                                                          \
                using Ids = mmc::dev::SmallRequests<mmc::dev::GpuIdsDefault>;                                          \
                __VA_ARGS__;                                                                                           \
            }                                                                                                          \
            else                                                                                                       \
            {                                                                                                          \
                using Ids = mmc::dev::GpuIdsDefault;                                                                   \
                __VA_ARGS__;                                                                                           \
            }                                                                                                          \
        }                                                                                                              \
        else                                                                                                           \
        {                                                                                                              \
            using Ids = mmc::dev::GpuIds;                                                                              \
            __VA_ARGS__;                                                                                               \
        }                                                                                                              \
    } while(0)

namespace mmc
{
    namespace host
    {
        /* Record msg as the calling thread's last error and return st. */
        mmc_status fail(mmc_status st, const std::string& msg);
        /* If e is an error: record it (with what) and return MMC_ERR_CUDA. */
        mmc_status cuda_check(cudaError_t e, const char* what);

        inline cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

        /* Grid for whole-heap scans: a multiple of the SM count. */
        unsigned scan_grid(int device);

        /* Launch the two-pass free-slot count of `slot` (already padded) and
         * leave the unsigned result in *result_dev (device memory). */
        mmc_status launch_available_slots(mmc_heap* heap, uint32_t slot, cudaStream_t s, unsigned* result_dev);

        /* Device-side word that receives the result of mmc_available_slots. */
        unsigned* slots_result_word(mmc_heap* heap);

        /* An NVTX range over a host entry point's work (heap set-up, slot
         * counts, launches of the batched and serving kernels), so Nsight
         * tools show each phase by name; without a tool attached it costs a
         * call into an empty stub. */
        struct NvtxRange
        {
            explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
            ~NvtxRange() { nvtxRangePop(); }
            NvtxRange(const NvtxRange&) = delete;
            NvtxRange& operator=(const NvtxRange&) = delete;
        };
    } // namespace host
} // namespace mmc

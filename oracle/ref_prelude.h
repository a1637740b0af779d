/* Compile prelude for building reference sources on alpaka's CPU-serial
 * backend without editing them (force-included with g++ -include):
 * 1. mallocMC_utils.hpp names alpaka::AccGpuUniformCudaHipRt, which alpaka only
 *    declares when a GPU backend is enabled; declare it for the CPU-only build.
 * 2. Scatter::calcAdditionalChunks calls alpaka::math::max/min with (int,
 *    unsigned). std::max cannot deduce that; CUDA's ::max/::min(int, unsigned)
 *    compare as unsigned, so these specialisations do the same.
 * TEST INFRASTRUCTURE ONLY (oracle/_ref). */
#pragma once
#include <alpaka/alpaka.hpp>

#include <algorithm>

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

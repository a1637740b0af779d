/* Minimal stand-in for <boost/core/demangle.hpp> built on the Itanium C++ ABI
 * demangler that g++ ships. Test infrastructure only. */
#pragma once
#include <cstdlib>
#include <cxxabi.h>
#include <string>

namespace boost
{
    namespace core
    {
        inline std::string demangle(char const* name)
        {
            int status = 0;
            char* out = abi::__cxa_demangle(name, nullptr, nullptr, &status);
            std::string s = (status == 0 && out) ? std::string(out) : std::string(name);
            std::free(out);
            return s;
        }
    } // namespace core
} // namespace boost

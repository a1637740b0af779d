/* Minimal stand-in for <boost/predef.h> for a g++ host-only build of the
 * reference's alpaka CPU backends. Only the macros alpaka tests are defined.
 * BOOST_COMP_MSVC_EMULATED / BOOST_COMP_PGI_EMULATED are deliberately left
 * undefined: alpaka tests them with defined(). Test infrastructure only. */
#pragma once
#include <boost/predef/version_number.h>

#if defined(__clang__)
#  define BOOST_COMP_CLANG BOOST_VERSION_NUMBER(__clang_major__, __clang_minor__, __clang_patchlevel__)
#  define BOOST_COMP_GNUC 0
#elif defined(__GNUC__)
#  define BOOST_COMP_CLANG 0
#  define BOOST_COMP_GNUC BOOST_VERSION_NUMBER(__GNUC__, __GNUC_MINOR__, __GNUC_PATCHLEVEL__)
#else
#  define BOOST_COMP_CLANG 0
#  define BOOST_COMP_GNUC 0
#endif
#define BOOST_COMP_NVCC 0
#define BOOST_COMP_MSVC 0
#define BOOST_COMP_PGI 0
#define BOOST_COMP_HPACC 0
#define BOOST_COMP_SUNPRO 0
#define BOOST_COMP_IBM 0
#define BOOST_LANG_CUDA 0
#define BOOST_ARCH_PTX 0
#if defined(__x86_64__) || defined(__i386__)
#  define BOOST_ARCH_X86 BOOST_VERSION_NUMBER_AVAILABLE
#else
#  define BOOST_ARCH_X86 0
#endif
#if defined(__linux__)
#  define BOOST_OS_LINUX BOOST_VERSION_NUMBER_AVAILABLE
#else
#  define BOOST_OS_LINUX 0
#endif
#if defined(__unix__) || defined(__unix)
#  define BOOST_OS_UNIX BOOST_VERSION_NUMBER_AVAILABLE
#else
#  define BOOST_OS_UNIX 0
#endif
#define BOOST_OS_MACOS 0
#define BOOST_OS_WINDOWS 0
#define BOOST_OS_CYGWIN 0
#define BOOST_OS_BSD 0
#define BOOST_PREDEF_MAKE_10_VVRRP(V) BOOST_VERSION_NUMBER(((V) / 1000) % 100, ((V) / 10) % 100, (V) % 10)
#define BOOST_PREDEF_MAKE_YYYYMMDD(V) BOOST_VERSION_NUMBER(((V) / 10000) % 10000 - 1970, ((V) / 100) % 100, (V) % 100)

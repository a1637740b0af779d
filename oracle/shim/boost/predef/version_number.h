/* Minimal stand-in for Boost.Predef's version-number macros, enough for the
 * reference's vendored alpaka headers to compile on a host-only (CPU) build.
 * Test infrastructure only: used to build the reference harness in oracle/_ref. */
#pragma once
#define BOOST_VERSION_NUMBER(major, minor, patch) \
    ((((major) % 100) * 10000000) + (((minor) % 100) * 100000) + ((patch) % 100000))
#define BOOST_VERSION_NUMBER_MAX BOOST_VERSION_NUMBER(99, 99, 99999)
#define BOOST_VERSION_NUMBER_ZERO BOOST_VERSION_NUMBER(0, 0, 0)
#define BOOST_VERSION_NUMBER_MIN BOOST_VERSION_NUMBER(0, 0, 1)
#define BOOST_VERSION_NUMBER_AVAILABLE BOOST_VERSION_NUMBER_MIN
#define BOOST_VERSION_NUMBER_NOT_AVAILABLE BOOST_VERSION_NUMBER_ZERO

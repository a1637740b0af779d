/* Minimal stand-in for <boost/version.hpp>. Test infrastructure only. */
#pragma once
#define BOOST_VERSION 108400
#define BOOST_LIB_VERSION "1_84"

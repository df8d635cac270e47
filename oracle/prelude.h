/*
 * Force-included compatibility prelude for compiling the unmodified reference
 * solver core (jak-xyz/xpbd-fem, XPBDFEM/*.cpp) headless with g++ on Linux.
 *
 * Test infrastructure only: used by oracle/build_ref.sh to build the golden
 * vector generator under oracle/_ref/. The reference was written for MSVC and a
 * wasm libc shim, both of which expose the float overloads of <cmath> in the
 * global namespace; glibc's <math.h> in C++ mode does not for all of them, so
 * they are pulled in here. Nothing in the reference is edited.
 */
#pragma once
#include <cstddef>
#include <cstdint>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <new>
#include <algorithm>
using std::abs; using std::acos; using std::acosh; using std::asin; using std::asinh;
using std::atan; using std::atanh; using std::ceil; using std::cos; using std::cosh;
using std::exp; using std::exp2; using std::floor; using std::log; using std::log2;
using std::round; using std::sin; using std::sinh; using std::sqrt; using std::tan;
using std::tanh; using std::trunc; using std::pow; using std::atan2; using std::fmod;
using std::fma; using std::modf;

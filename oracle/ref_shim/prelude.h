// Forced-include prelude for compiling the reference's MSVC-flavoured headers
// with g++ on Linux (x86_64 or aarch64).  Test infrastructure only.
//  - standard headers MSVC pulls in transitively;
//  - `sprintf_s`, used by stb_image_write because `Imaging.h:15` defines
//    `__STDC_LIB_EXT1__`;
//  - `std::cosf`-style names used by `Materials.h:700-702,809-817` that
//    libstdc++ does not declare in namespace std.
#pragma once
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>

#define sprintf_s snprintf

namespace std {
using ::cosf;
using ::powf;
using ::sinf;
using ::sqrtf;
using ::tanf;
}  // namespace std

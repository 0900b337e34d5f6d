// Stand-in for Boost.Math sign functions (dax/math/Sign.h:32). Test infrastructure only.
#pragma once
#include <cmath>
namespace boost { namespace math { using std::signbit; using std::copysign; } }

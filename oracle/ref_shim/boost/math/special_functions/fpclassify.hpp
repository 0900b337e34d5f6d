// Stand-in for Boost.Math classification (dax/math/Precision.h:36). Test infrastructure only.
#pragma once
#include <cmath>
namespace boost { namespace math { using std::isnan; using std::isinf; using std::isfinite; } }

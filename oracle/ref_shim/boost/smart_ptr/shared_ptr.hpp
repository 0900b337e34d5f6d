// Stand-in for boost::shared_ptr (dax/cont/ArrayHandle.h:28). Test infrastructure only.
#pragma once
#include <memory>
namespace boost { using std::shared_ptr; }

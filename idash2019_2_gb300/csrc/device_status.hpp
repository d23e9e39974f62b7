// Codes a kernel writes into the context's device error word (first wins).
#pragma once

#include <cstdint>

namespace idash {

enum : uint32_t {
    kDevOk = 0,
    kDevTimeout = 1,   // an mbarrier wait ran past its cycle limit
    kDevBadIndex = 2,  // a plan entry pointed outside its buffer
};

}  // namespace idash

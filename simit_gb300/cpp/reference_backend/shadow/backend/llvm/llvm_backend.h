// Used in place of the reference's LLVM backend header when the reference's
// backend factory (src/backend/backend.cpp:20-33) is compiled into this
// repository's link of the reference, which has no LLVM: the backend that
// the factory constructs for the default type "cpu" is the GB300 backend.
// A maintainer adding the backend to the reference tree instead adds a
// "gb300" branch to that factory and to VALID_BACKENDS (src/program.cpp:
// 20-25), next to the "gpu" ones.
#pragma once
#include "../../../gb300_backend.h"

namespace simit {
namespace backend {
typedef GB300Backend LLVMBackend;
}  // namespace backend
}  // namespace simit

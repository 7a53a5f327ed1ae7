// oracle/ref/ref_shim.hpp -- TEST INFRASTRUCTURE ONLY.
//
// Force-included (g++ -include) into every reference C++ translation unit the
// oracle recipe compiles. It works around two defects that stop the reference
// from compiling as shipped, without editing its sources:
//   1. include/vibe/common/logging.hpp:63-70 names the VIBE_LOG macro parameter
//      `level`, which also rewrites the `.level()` call inside the macro body.
//      The macro is redefined here with a parameter name that does not clash.
//   2. src/time/helmholtz.cpp:431 uses an unqualified `Precision`; only
//      vibe::gpu::Precision exists (include/vibe/time/helmholtz.hpp:85).
#pragma once
#include "vibe/common/logging.hpp"

#undef VIBE_LOG
#define VIBE_LOG(lvl_, ...)                                                  \
  do {                                                                       \
    if (static_cast<int>(lvl_) >=                                            \
        static_cast<int>(::vibe::common::Logger::instance().level())) {      \
      ::vibe::common::Logger::instance().write(                              \
          lvl_, ::vibe::common::detail::format(__VA_ARGS__));                \
    }                                                                        \
  } while (false)

#include "vibe/gpu/precision.hpp"
namespace vibe::timeint {
using vibe::gpu::Precision;
}

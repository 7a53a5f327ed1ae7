// oracle/ref/ref_odr_fix.cpp -- TEST INFRASTRUCTURE ONLY.
//
// include/vibe/dyn/advection.hpp:36 declares advection_from_string `inline`
// while src/dyn/advection.cpp:36-42 defines it out of line, so no external
// definition is emitted and equations.o fails to link. This translation unit
// does not include advection.hpp; it declares the enum with the same
// enumerators (advection.hpp:34) and emits one external definition with the
// same mapping as advection.cpp:36-42.
#include <string>

namespace vibe::dyn {
enum class AdvectionScheme { Central2, Central4, Central6, WENO5, Upwind3 };

AdvectionScheme advection_from_string(const std::string& s) {
  if (s == "central4") return AdvectionScheme::Central4;
  if (s == "central6") return AdvectionScheme::Central6;
  if (s == "weno5") return AdvectionScheme::WENO5;
  if (s == "upwind3") return AdvectionScheme::Upwind3;
  return AdvectionScheme::Central2;
}
}  // namespace vibe::dyn

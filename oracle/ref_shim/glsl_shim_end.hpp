// glsl_shim_end.hpp -- ends the shader section of the translation unit:
// removes the qualifier macros of glsl_shim.hpp before the driver code.
#pragma once
#undef in
#undef out
#undef inout
#undef flat
#undef uniform
#undef layout
#undef discard
#undef mat3

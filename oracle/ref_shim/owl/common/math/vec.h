// Stand-in for the absent OWL header of the same name (reference host shim).
#pragma once
#include "../../../hm_owl_shim.h"
// the terminal colour escapes of OWL's common header, used by the
// reference's LOG macros (no colours here)
#define OWL_TERMINAL_BLUE ""
#define OWL_TERMINAL_LIGHT_BLUE ""
#define OWL_TERMINAL_DEFAULT ""

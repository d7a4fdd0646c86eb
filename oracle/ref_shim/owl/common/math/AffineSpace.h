// Stand-in for the absent OWL header of the same name (reference host shim).
#pragma once
#include "../../../hm_owl_shim.h"

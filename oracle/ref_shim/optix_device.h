// Stand-in for OptiX's device header on the host build: everything the
// reference's programs use from it is provided by hm_owl_shim.h.
#pragma once
#include "hm_owl_shim.h"

// OpenEXR environment-map reader (hm_exr.cu).
#pragma once
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace hm {

// Decodes a single-part scanline OpenEXR file held in `data` into RGBA float
// rows (first stored line first), as tinyexr's LoadEXR returns them.
// HM_OK, HM_EPARSE (malformed) or HM_EUNSUPPORTED (a layout or compression
// this reader does not decode), with the reason in *err.
int exr_load_rgba(const std::string& data, std::vector<float4>* rgba, int* width, int* height, std::string* err);

}  // namespace hm

// The reference's scene.cpp (parseScene, Scene::extractHairData,
// LoadCemYuksel, generateEnvSamplingTables), compiled unmodified on the host
// (test infrastructure only; built by oracle/build.py into oracle/_ref/,
// never committed, never shipped).  Its absent dependencies are stand-ins in
// this folder: OWL's vector headers (hm_owl_shim.h), cyHairFile.h (Cem
// Yuksel's HAIR reader) and json/json.hpp (nlohmann::json).  The OBJ and EXR
// loaders of model.cpp are not built: loadOBJ returns an empty model and
// loadEnvTexture does nothing, so parseScene's surface / environment
// branches run without reading those files.
#include "scene.cpp"

#include <cstring>

Model* loadOBJ(const std::string&) { return new Model(); }
bool loadEnvTexture(std::string&, Texture*) { return true; }

extern "C" {

// generateEnvSamplingTables (scene.cpp:349-425) on an RGBA float map
// [h][w][4]: cpdf / ccdf [h][w + 1], mpdf / mcdf [h + 1].
void hmr_env_tables(int w, int h, const float* env4, float* cpdf, float* ccdf, float* mpdf, float* mcdf) {
  float *cp = nullptr, *cc = nullptr, *mp = nullptr, *mc = nullptr;
  generateEnvSamplingTables(vec2i(w, h), const_cast<float*>(env4), &cp, &cc, &mp, &mc);
  memcpy(cpdf, cp, sizeof(float) * (size_t)(w + 1) * h);
  memcpy(ccdf, cc, sizeof(float) * (size_t)(w + 1) * h);
  memcpy(mpdf, mp, sizeof(float) * (size_t)(h + 1));
  memcpy(mcdf, mc, sizeof(float) * (size_t)(h + 1));
  free(cp);
  free(cc);
  free(mp);
  free(mc);
}

// LoadCemYuksel + Scene::extractHairData (scene.cpp:10-117) on a HAIR file.
// Returns the number of control points (-1 if the file does not load) and
// fills, up to the capacities: cp [n][4] (x, y, z, width), seg [m]
// (segmentIndices), info [3] (control points, segments, strands) and
// bounds [7] (minBound, maxBound, scale).
int hmr_hair_file(const char* path, float* cp, int cap_cp, int* seg, int cap_seg, int* info, float* bounds) {
  Scene s;
  if (s.hair.LoadFromFile(path) < 0) return -1;
  LoadCemYuksel(path, s.hair);
  s.extractHairData();
  const HairModel& m = s.hairModel;
  const int n = (int)m.controlPoints.size(), k = (int)m.segmentIndices.size();
  for (int i = 0; i < n && i < cap_cp; ++i) {
    cp[4 * i] = m.controlPoints[i].x;
    cp[4 * i + 1] = m.controlPoints[i].y;
    cp[4 * i + 2] = m.controlPoints[i].z;
    cp[4 * i + 3] = m.widths[i];
  }
  for (int i = 0; i < k && i < cap_seg; ++i) seg[i] = m.segmentIndices[i];
  info[0] = n;
  info[1] = k;
  info[2] = m.numStrands;
  const float b[7] = {m.minBound.x, m.minBound.y, m.minBound.z, m.maxBound.x, m.maxBound.y, m.maxBound.z, m.scale};
  memcpy(bounds, b, sizeof(b));
  return n;
}

// parseScene (scene.cpp:119-339) on a scene file.  Returns its result (1 /
// 0; -1 when the JSON text itself does not parse, which the reference does
// not catch).  vals [40]: camera from, at, up, cosFovy (10); bsdf; sig_a (3);
// beta_m, beta_n, alpha; R, TT, TRT, TRRT gains; pixarFactor; hasEnvLight,
// envScale, envRotPhi; hasDirectionalLights, number of directional lights;
// MIS, envPdfSampling; spp, path_v1, path_v2, imgWidth, imgHeight;
// nrcTrain; has_hair, has_surface (39 used).  lights [8][6]: the first
// directional lights' from (normalized) and emit.  text: renderOutput,
// renderStatsOutput, nrcConfig, nrcConfig2, nrcWeights,
// dualScatterPrecompPath, each NUL-terminated, packed.
int hmr_parse_scene(const char* path, float* vals, float* lights, char* text, int text_cap) {
  Scene s;
  bool ok = false;
  try {
    ok = parseScene(path, s);
  } catch (const nlohmann::json::exception&) {
    return -1;
  }
  const float v[39] = {s.camera.from.x, s.camera.from.y, s.camera.from.z, s.camera.at.x, s.camera.at.y,
                       s.camera.at.z, s.camera.up.x, s.camera.up.y, s.camera.up.z, s.camera.cosFovy,
                       (float)s.bsdf, s.sig_a.x, s.sig_a.y, s.sig_a.z, s.beta_m, s.beta_n, s.alpha, s.R_G, s.TT_G,
                       s.TRT_G, s.TRRT_G, s.pixarFactor, s.hasEnvLight ? 1.f : 0.f, s.envScale, s.envRotPhi,
                       s.hasDirectionalLights ? 1.f : 0.f, (float)s.dLightFrom.size(), s.MIS ? 1.f : 0.f,
                       s.envPdfSampling ? 1.f : 0.f, (float)s.spp, (float)s.path_v1, (float)s.path_v2,
                       (float)s.imgWidth, (float)s.imgHeight, s.nrcTrain ? 1.f : 0.f, s.has_hair ? 1.f : 0.f,
                       s.has_surface ? 1.f : 0.f, 0.f, 0.f};
  memcpy(vals, v, sizeof(v));
  for (size_t i = 0; i < s.dLightFrom.size() && i < 8; ++i) {
    const float l[6] = {s.dLightFrom[i].x, s.dLightFrom[i].y, s.dLightFrom[i].z,
                        s.dLightEmit[i].x, s.dLightEmit[i].y, s.dLightEmit[i].z};
    memcpy(lights + 6 * i, l, sizeof(l));
  }
  std::string packed;
  for (const std::string* t : {&s.renderOutput, &s.renderStatsOutput, &s.nrcConfig, &s.nrcConfig2, &s.nrcWeights,
                               &s.dualScatterPrecompPath}) {
    packed += *t;
    packed += '\0';
  }
  if ((int)packed.size() <= text_cap) memcpy(text, packed.data(), packed.size());
  if (s.surface && s.has_surface) delete s.surface;
  return ok ? 1 : 0;
}

}  // extern "C"

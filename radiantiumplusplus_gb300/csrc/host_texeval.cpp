// Host evaluation of the scene's textures with the device code (dtex.cuh built
// for the host): the scene builder reads textures where the reference reads
// them at build time (the skybox luminance grid, skybox.cpp:27-47), so the
// host and device lookups are the same arithmetic.
#define RAD_HOST_EMULATION 1
#include "dtex.cuh"
#include "host_scene.h"

namespace rad {

void HostTexEval(const HostScene& hs, uint32_t tex, float u, float v, float out[3]) {
  TexCtx x{hs.tex.data(), hs.texels.data(), hs.texBind.data(), V2{u, v}, V2{0.f, 0.f}, V2{0.f, 0.f}};
  TexVal r = TexEval(x, tex, x.uv);
  out[0] = r.c[0];
  out[1] = r.c[1];
  out[2] = r.c[2];
}

}  // namespace rad

// pbr_hard_tex.cu -- the tile kernel with texture sampling (textured nodes,
// shaders/basic.frag:31-32), a translation unit of its own so that the
// untextured instantiations in pbr_hard.cu keep their register allocation and
// the two compile in parallel.
#include "pbr_hard.cuh"
#include "pbr_launch.h"

namespace pbr {

template <int T, bool PL, bool WN>
static const void* tex_fn() {
  return reinterpret_cast<const void*>(&hard_kernel<T, PL, WN, true>);
}

const void* hard_tex_fn(int threads, bool plain, bool winner) {
  if (plain) {
    if (winner) return nullptr;
    switch (threads) {
      case 128: return tex_fn<128, true, false>();
      case 256: return tex_fn<256, true, false>();
      case 512: return tex_fn<512, true, false>();
    }
    return nullptr;
  }
  switch (threads) {
    case 128: return winner ? tex_fn<128, false, true>() : tex_fn<128, false, false>();
    case 256: return winner ? tex_fn<256, false, true>() : tex_fn<256, false, false>();
    case 512: return winner ? tex_fn<512, false, true>() : tex_fn<512, false, false>();
  }
  return nullptr;
}

}  // namespace pbr

// fftreg_f32.cu — register-resident FFT passes instantiated for float (see fftreg_impl.cuh).
#include "fftreg_impl.cuh"

namespace ttsh {

template <>
bool fftreg_launch<float>(const Group<float>& g, int pass, cudaStream_t st) {
  return g.fft_kind != 1 && fftreg::reg_launch<float>(g, pass, st);
}
template <>
bool fftreg_plane_launch<float>(const Group<float>& g, int dir, cudaStream_t st) {
  return g.fft_kind == 2 && fftreg::reg_plane_launch<float>(g, dir, st);
}
template <>
bool fftreg_has<float>(int N) {
  return fftreg::reg_supported<float>(N);
}
template <>
void fftreg_prepare<float>(int N) {
  fftreg::reg_prepare<float>(N);
}

}  // namespace ttsh

// fftreg_f64.cu — register-resident FFT passes instantiated for double (see fftreg_impl.cuh).
#include "fftreg_impl.cuh"

namespace ttsh {

template <>
bool fftreg_launch<double>(const Group<double>& g, int pass, cudaStream_t st) {
  return g.fft_kind != 1 && fftreg::reg_launch<double>(g, pass, st);
}
template <>
bool fftreg_plane_launch<double>(const Group<double>& g, int dir, cudaStream_t st) {
  return g.fft_kind == 2 && fftreg::reg_plane_launch<double>(g, dir, st);
}
template <>
bool fftreg_has<double>(int N) {
  return fftreg::reg_supported<double>(N);
}
template <>
void fftreg_prepare<double>(int N) {
  fftreg::reg_prepare<double>(N);
}
template <>
void fftreg_twiddles<double>(int N) {
  fftreg::reg_twiddles<double>(N);
}

}  // namespace ttsh

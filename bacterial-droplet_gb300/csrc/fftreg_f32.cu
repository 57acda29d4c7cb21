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
template <>
void fftreg_twiddles<float>(int N) {
  fftreg::reg_twiddles<float>(N);
}

int fftreg_zt_setup(int N, const std::vector<const void*>& W, void** d_maps) {
  *d_maps = nullptr;
  const int grid = fftreg::reg_zt_prepare(N);
  if (grid <= 0 || W.empty()) return 0;
  std::vector<CUtensorMap> maps(W.size());
  for (size_t i = 0; i < W.size(); ++i) fftreg::reg_zt_encode(N, W[i], &maps[i]);
  void* d = nullptr;
  cudaError_t e = cudaMalloc(&d, maps.size() * sizeof(CUtensorMap));
  if (e == cudaSuccess) e = cudaMemcpy(d, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (d) cudaFree(d);
    throw std::runtime_error(std::string("fft (staged z) descriptors: ") + cudaGetErrorString(e));
  }
  *d_maps = d;
  return grid;
}

}  // namespace ttsh

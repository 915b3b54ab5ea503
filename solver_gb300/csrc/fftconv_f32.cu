// float instantiation of the circulant convolution passes (fftconv_impl.cuh).
#include "fftconv_impl.cuh"

namespace peec {

int conv_all_f32(const Family* F, int nfam, const Spectrum* spec, const void* const* ph,
                 const c64* x, c64* LpI, c64* PQ, int64_t m, const void* tw, int twmax,
                 cudaStream_t st, cudaEvent_t* ev, const ZTune* zt) {
  return conv_all_t<float>(F, nfam, spec, ph, x, LpI, PQ, m, reinterpret_cast<const c32*>(tw),
                        twmax, st, ev, zt);
}

int zpass_f32(const Family* F, int nfam, const Spectrum* spec, const void* const* ph,
              const void* tw, int twmax, const ZTune& zt, int which, cudaStream_t st) {
  const PSpec S = pspec_of<float>(spec, ph);
  if (which == 0) return zface_f32(F, nfam, S, reinterpret_cast<const c32*>(tw), twmax, zt, st);
  return zedge_f32(F, nfam, spec, reinterpret_cast<const c32*>(tw), twmax, zt, st);
}

}  // namespace peec

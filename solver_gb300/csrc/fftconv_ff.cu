// ff instantiation of the circulant convolution passes (fftconv_impl.cuh).
#include "fftconv_impl.cuh"

namespace peec {

int conv_all_ff(const Family* F, int nfam, const Spectrum* spec, const void* const* ph,
                 const c64* x, c64* LpI, c64* PQ, int64_t m, const void* tw, int twmax,
                 cudaStream_t st, cudaEvent_t* ev, const ZTune* zt) {
  return conv_all_t<ff>(F, nfam, spec, ph, x, LpI, PQ, m, reinterpret_cast<const cff*>(tw),
                        twmax, st, ev, zt);
}

}  // namespace peec

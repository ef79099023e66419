// wave_r26.cu -- batched-form kernels with 26 rows per lane (bands of 208, 416 or 832 rows).
#include "wave_impl.cuh"

namespace nwg {
NWG_DEFINE_WAVE(26)
}  // namespace nwg

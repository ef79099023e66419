// wave_r18.cu -- batched-form kernels with 18 rows per lane (bands of 144, 288 or 576 rows).
#include "wave_impl.cuh"

namespace nwg {
NWG_DEFINE_WAVE(18)
}  // namespace nwg

// wave_r30.cu -- batched-form kernels with 30 rows per lane (bands of 240, 480 or 960 rows).
#include "wave_impl.cuh"

namespace nwg {
NWG_DEFINE_WAVE(30)
}  // namespace nwg

// wave_r28.cu -- batched-form kernels with 28 rows per lane (bands of 224, 448 or 896 rows).
#include "wave_impl.cuh"

namespace nwg {
NWG_DEFINE_WAVE(28)
}  // namespace nwg

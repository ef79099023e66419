// wave_r22.cu -- batched-form kernels with 22 rows per lane (bands of 176, 352 or 704 rows).
#include "wave_impl.cuh"

namespace nwg {
NWG_DEFINE_WAVE(22)
}  // namespace nwg

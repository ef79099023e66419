// wave_r32.cu -- batched-form kernels with 32 rows per lane (band of 1024 rows).
#include "wave_impl.cuh"

namespace nwg {
NWG_DEFINE_WAVE(32)
}  // namespace nwg

/* Host stand-in: the reference's kernel text includes <cuda.h>; the host build of
 * that text (oracle/ref_shim/ref_kernels.cpp) needs only the vector types. */
#include "vector_types.h"

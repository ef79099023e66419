/* Host stand-in for the CUDA vector types the reference's kernel text uses
 * (short2, char2, uint3, dim3).  Test infrastructure only: lets a host
 * compiler build NeedlemanWunsch.cu's kernels one pair at a time
 * (oracle/ref_shim/ref_kernels.cpp). */
#ifndef NWG_SHIM_VECTOR_TYPES_H
#define NWG_SHIM_VECTOR_TYPES_H
struct short2 { short x, y; };
struct char2 { signed char x, y; };
struct uint3 { unsigned int x, y, z; };
struct dim3 { unsigned int x, y, z; };
#endif

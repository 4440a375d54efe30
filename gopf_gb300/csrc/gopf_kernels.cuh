// gopf_kernels.cuh -- launch interface of the spectral-step kernels.
//
// Spectral layout in HBM (ours, not the reference's): a real field of the
// reference's domainSize [n0 rows, n1 cols, n2 depth] (node index
// depth*n0*n1 + row*n1 + col, pfutil/indexPositionConversion.go:23-34) is kept
// as its half spectrum S[z][kx][y] with kx in [0, n1/2] slowest inside a
// depth plane and the row frequency y fastest.  Every pass then reads either
// whole contiguous lines (the y axis) or 128-byte segments of LB consecutive
// y values (the kx and z axes).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "fft_core.cuh"
#include "gopf_types.h"

namespace gopf {
// Launchers (return cudaError_t of the launch)
template <typename R> cudaError_t launch_xpass(const XPassArgs<R> &a, int LB, cudaStream_t st);
// number of FP64 partial-sum rows launch_xpass writes to a.red for this launch
template <typename R> int xpass_red_blocks(const XPassArgs<R> &a, int LB);
template <typename R> cudaError_t launch_cpass(const PassArgs<R> &a, int LB, cudaStream_t st); // contiguous y axis
template <typename R> cudaError_t launch_spass(const PassArgs<R> &a, int LB, cudaStream_t st); // strided z axis

// Tile width (lines per tile) for a transform of length n: 128 bytes per tile
// row where the 256-thread block can hold LB*n/16 butterfly inputs.
inline int lb_for(int n, int vbytes)
{
    int lb = 128 / vbytes;
    while (lb > 4 && lb * n > 4096) lb /= 2;
    return lb;
}
inline int xpass_smem_bytes(const Geom &g, int LB, int vbytes, int ntiles = 2);
inline int cpass_smem_bytes(const Geom &g, int n, int LB, int nbuf, int vbytes);
inline int spass_smem_bytes(const Geom &g, int n, int LB, int nbuf, int vbytes);

} // namespace gopf

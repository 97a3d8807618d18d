// Launch wrappers for the point-layout conversions (see state_io.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fgb {

template <class T>
cudaError_t launch_unpack(int n, const float* pts, const uint8_t* pinned, void* pos, void* vel, void* force,
                          cudaStream_t s);
template <class T>
cudaError_t launch_pack_f32(int n, const void* pos, const void* vel, const void* force, float* pts, cudaStream_t s);
template <class T>
cudaError_t launch_pack_f64(int n, const void* pos, const void* vel, const void* force, double* pts,
                            cudaStream_t s);
template <class T>
cudaError_t launch_positions(int n, const void* pos, float* out, cudaStream_t s);
template <class T>
cudaError_t launch_set_pins(int n, const uint8_t* pinned, void* vel, cudaStream_t s);

}  // namespace fgb

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

// Render vertices (graphics/model.rs:170-186, ColoredVertex = position,
// color, normal: 9 f32 per vertex) straight from the device state; the normal
// of vertex v is the sum, in face order, of (p_a - p_b) x (p_a - p_c) over its
// faces (a, b, c), normalised (graphics/util.rs:178-199).  face_off/face_inc
// are the general CSR lists (face<<2|corner, ascending face id), face_vtx 4
// ints per face.
template <class T>
cudaError_t launch_render_vertices(int n, const void* pos, const int* face_off, const int* face_inc,
                                   const int4* face_vtx, float r, float g, float b, float* out, cudaStream_t s);

}  // namespace fgb

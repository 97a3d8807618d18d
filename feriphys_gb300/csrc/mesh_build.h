// Host-side mesh construction with the reference's semantics and ordering
// (SpringyMesh::new springy_mesh.rs:267-401, add_strut 403-413, add_pin
// 415-417, Cloth::new cloth.rs:20-113), plus the device-layout builders:
// CSR incidence lists for the general gather and the owned-strut parameter
// planes for the grid stencil kernel.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "grid_order.h"

namespace fgb {

struct MeshTopo {
  uint32_t n = 0;
  std::vector<float> pos;  // 3n, positions used for rest lengths (construction time)
  float mass_per_vert = 0.0f;
  // struts in reference order
  std::vector<uint32_t> sa, sb;
  std::vector<float> sk, sc, sl;
  // faces in reference order
  std::vector<uint32_t> fv;  // 3 per face
  std::vector<uint32_t> fs;  // 3 per face (strut ids)
  std::vector<uint32_t> pins;
  // set when the triangle list is exactly Cloth::new's for rows x cols
  uint32_t rows = 0, cols = 0;
  size_t tri_struts = 0;  // struts created from the triangle list
};

struct Override {
  uint32_t a, b;
  float k, c;
};

// Returns 0 or a negative fgb_status; err gets a message.
int build_springy(const float* pos, uint64_t nv, const uint32_t* idx, uint64_t ni, float mass, float k, float c,
                  const Override* ov, uint64_t nov, MeshTopo& out, std::string& err);
int build_cloth(uint64_t rows, uint64_t cols, float spacing, const float position[3], float point_mass, float tk,
                float tc, float sk, float sc, float bk, float bc, const uint32_t* pins, uint64_t npins,
                MeshTopo& out, std::string& err);
// The same result as build_springy with the strut de-duplication, the
// face/strut adjacency and the strut constants computed on the current GPU
// (mesh_build_gpu.cu); identical output, including error codes and messages.
int build_springy_device(const float* pos, uint64_t nv, const uint32_t* idx, uint64_t ni, float mass, float k,
                         float c, const Override* ov, uint64_t nov, MeshTopo& out, std::string& err);
// True when the triangle list is exactly Cloth::new's for some rows x cols.
bool detect_cloth_pattern(const uint32_t* idx, uint64_t nt, uint32_t n, uint32_t& R, uint32_t& C);
// add_strut: rest length from the points' current positions, read at
// cur_pos[stride * i + 0..2].
int add_strut(MeshTopo& m, uint32_t a, uint32_t b, float k, float c, const float* cur_pos, size_t stride,
              std::string& err);

// Strut::new's length scaling: NOMINAL_STRUT_LENGTH / length * nominal (springy_mesh.rs:83-84).
inline float scaled(float nominal, float length) { return 1.0f / length * nominal; }

// Duration::from_secs_f32(x).as_secs_f32() with modern Rust's rounding to
// whole nanoseconds (nearest, ties to even).  x finite and >= 0.
float duration_roundtrip(float x);
// Duration::from_secs_f32(x).as_secs_f64().
double duration_seconds_f64(float x);

// CSR incidence lists for the general gather (see step_general.cu).
struct CsrTopo {
  std::vector<int> strut_off;       // n+1
  std::vector<int> strut_inc;       // 2 per entry: other, strut<<1|role
  std::vector<float> strut_kcl;     // 4 per strut
  std::vector<int> face_off;        // n+1
  std::vector<int> face_inc;        // face<<2|corner
  std::vector<int> face_vtx;        // 4 per face
};
int build_csr(const MeshTopo& m, CsrTopo& out, std::string& err);

// The compact form of the same incidence lists (see step_general.cu), which
// the step reads instead of strut_inc, strut_kcl, face_inc and face_vtx:
//   own_off[v]..own_off[v+1]   the struts whose first vertex is v, ascending
//                              by strut id ("owner order")
//   sk/sc/sl[i]                stiffness, damping, rest length of the strut
//                              at owner position i
//   strut_word[e]              per strut incidence (same order and offsets as
//                              strut_inc): (other - v) << 6 | rank << 1 | role,
//                              rank = the strut's position in its first
//                              vertex's owner range; or, when they fit,
//   strut_word16[e]            the same in 16 bits (strut_word stays empty):
//                              role 0: (other - v) << 1, the offset in
//                              [-16384, 16383] (no rank: v's own struts are
//                              taken in order); role 1: (other - v) << 4 |
//                              rank << 1 | 1, the offset in [-2048, 2047] and
//                              the rank below 8
//   face_word[e]               per face incidence (same order and offsets as
//                              face_inc): corner | i1 << 2 | i2 << 9, i1 and i2
//                              the positions in v's strut list of the face's
//                              other two vertices, in face order
// Returns false (and leaves out empty) when the mesh does not fit it: a face
// vertex that is no strut neighbour, a vertex with more than 127 strut
// incidences, more than 32 struts owned by one vertex, or a vertex offset
// beyond +-2^25.
struct CompactTopo {
  std::vector<int> own_off;             // n+1
  std::vector<float> sk, sc, sl;        // S each, owner order
  std::vector<uint32_t> strut_word;     // one per strut incidence (32-bit form)
  std::vector<uint16_t> strut_word16;   // one per strut incidence (16-bit form)
  std::vector<uint16_t> face_word;      // one per face incidence
};
bool build_compact(const MeshTopo& m, const CsrTopo& t, CompactTopo& out);

// Grid detection: true when the mesh is Cloth::new's rows x cols grid with
// exactly its binding struts after the triangle struts, and the strut ids
// around every vertex ascend in the order the grid kernel sums them.
bool grid_layout_ok(const MeshTopo& m);
// Owned-strut constants, 4 float4 planes of n entries (see grid_order.h).
void build_grid_params(const MeshTopo& m, std::vector<float>& planes /*16*n*/);

}  // namespace fgb

// Neighbourhood of a vertex in a Cloth::new grid, in the order the reference
// sums its force terms.  Shared by the host (which checks the order against
// the actual strut and face ids before using the grid kernel) and the
// device (which sums in this order).
//
// Cloth::new (cloth.rs:63-110) builds, for quad q = (r, c) with origin
// i = r*C + c:
//   face A(q) = (i+1, i+C, i)       first pass, face id q
//   face B(q) = (i+1, i+C+1, i+C)   second pass, face id (R-1)(C-1) + q
// SpringyMesh::new de-duplicates the edges in that order, so every quad
// first creates  shear (i+1, i+C), vertical (i, i+C), horizontal (i, i+1);
// the second pass adds the last column's verticals and the last row's
// horizontals; the binding struts (i, i+2), (i, i+2C) come last.
//
// Each strut is "owned" by one vertex whose parameter slot holds its
// constants: horizontal and vertical and binding struts by their first
// vertex, a shear strut (i+1, i+C) by its quad origin i.
#pragma once

#if defined(__CUDACC__)
#define FGB_HD __host__ __device__ __forceinline__
#else
#define FGB_HD inline
#endif

namespace fgb {
namespace grid {

enum Kind { KH = 0, KV = 1, KS = 2, KBH = 3, KBV = 4 };

// Strut slots around a vertex.
enum Slot { SH_UP = 0, VT_UP, SH_LEFT, HZ_LEFT, VT_DOWN, HZ_RIGHT, BV_UP, BH_LEFT, BH_RIGHT, BV_DOWN, N_SLOTS };

struct SlotDesc {
  int dr, dc;  // owner = (r + dr, c + dc)
  int kind;
  int role;  // 0: this vertex is the strut's first vertex, 1: its second
};

FGB_HD SlotDesc slot_desc(int s) {
  switch (s) {
    case SH_UP: return {-1, 0, KS, 1};
    case VT_UP: return {-1, 0, KV, 1};
    case SH_LEFT: return {0, -1, KS, 0};
    case HZ_LEFT: return {0, -1, KH, 1};
    case VT_DOWN: return {0, 0, KV, 0};
    case HZ_RIGHT: return {0, 0, KH, 0};
    case BV_UP: return {-2, 0, KBV, 1};
    case BH_LEFT: return {0, -2, KBH, 1};
    case BH_RIGHT: return {0, 0, KBH, 0};
    default: return {0, 0, KBV, 0};  // BV_DOWN
  }
}

// Does the strut of `kind` owned by (r, c) exist in an R x C cloth?
FGB_HD bool owned_exists(int kind, int r, int c, int R, int C) {
  if (r < 0 || c < 0) return false;
  switch (kind) {
    case KH: return c <= C - 2 && r <= R - 1;
    case KV: return r <= R - 2 && c <= C - 1;
    case KS: return r <= R - 2 && c <= C - 2;
    default: return r <= R - 3 && c <= C - 3;  // binding struts (cloth.rs:101-107)
  }
}

// The j-th strut slot of vertex (r, c) in summation order.  The last
// column's upward vertical is created by the second triangle pass, after
// the shear and horizontal struts of its row, so it moves behind them.
FGB_HD int slot_at(int j, int r, int c, int R, int C) {
  const bool late_vertical = (c == C - 1) && r >= 1 && r <= R - 2;
  if (!late_vertical) return j;
  if (j == VT_UP) return SH_LEFT;
  if (j == SH_LEFT) return HZ_LEFT;
  if (j == HZ_LEFT) return VT_UP;
  return j;
}

// Face slots around a vertex (faces sum after all struts, in this order).
enum FaceSlot { A_UP = 0, A_LEFT, A_HERE, B_UPLEFT, B_UP, B_LEFT, N_FACE_SLOTS };

struct FaceDesc {
  int dr, dc;  // quad = (r + dr, c + dc)
  int is_b;    // 0: face A(q), 1: face B(q)
  int corner;  // this vertex's corner in the face's vertex triple
};

FGB_HD FaceDesc face_desc(int s) {
  switch (s) {
    case A_UP: return {-1, 0, 0, 1};
    case A_LEFT: return {0, -1, 0, 0};
    case A_HERE: return {0, 0, 0, 2};
    case B_UPLEFT: return {-1, -1, 1, 1};
    case B_UP: return {-1, 0, 1, 2};
    default: return {0, -1, 1, 0};  // B_LEFT
  }
}

FGB_HD bool quad_exists(int r, int c, int R, int C) { return r >= 0 && c >= 0 && r <= R - 2 && c <= C - 2; }

// Parameter plane layout: 4 float4 per vertex, 15 used floats.
//   plane 0: kH  cH  LH  kV
//   plane 1: cV  LV  kS  cS
//   plane 2: LS  kBH cBH LBH
//   plane 3: kBV cBV LBV -
FGB_HD int param_index(int kind, int field /*0 k, 1 c, 2 L*/) { return 3 * kind + field; }

}  // namespace grid
}  // namespace fgb

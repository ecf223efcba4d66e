// Oracle-side dual-marching-cubes tables (test infrastructure, not shipped).
//
// Two tables drive the reference's dual-cell triangulation:
//  * the 256-entry canonicalisation table `table[256]`
//    (reference include/visitorextract.h:35-293): for every 8-bit corner-sign
//    code, a corner permutation `trans`, an orientation `flip` and the
//    canonical code of its symmetry class;
//  * the triangle list of each of the 20 non-trivial canonical codes
//    (reference src/visitorextract.cpp:95-199), and the edge -> corner map
//    `dual_edge2vert` (include/visitorextract.h:306-311).
//
// The canonicalisation table is not copied: it is regenerated from a rule.
// Every entry maps the code to the minimum of its orbit under the 48 cube
// symmetries (no complement); the symmetry chosen is the first that reaches the
// minimum when symmetries are enumerated xor-mask-major (mask 0..7) and, inside
// a mask, over the axis permutations in the order listed in kPermOrder; flip is
// set for orientation-reversing symmetries.  A CPU test checks the generated
// table against a digest of the reference table.
//
// The triangle lists cannot be derived (they fix diagonal choices and winding)
// and must be identical for mesh parity, so they are restated here as data in a
// compact form: per canonical code, a string of edge indices in hex, three per
// triangle.
#pragma once
#include <cstdint>
#include <cstring>

namespace pio {

struct DmcProc {
  int trans[8];
  bool flip;
  int code;
};

// Axis permutations in enumeration order; perm[k] is the bit that corner bit k
// moves to.
static const int kPermOrder[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2},
                                     {1, 2, 0}, {2, 1, 0}, {2, 0, 1}};

inline void dmc_symmetry(int perm_idx, int mask, int trans[8], bool* reflect) {
  const int* p = kPermOrder[perm_idx];
  for (int i = 0; i < 8; ++i) {
    int o = 0;
    for (int k = 0; k < 3; ++k) o |= ((i >> k) & 1) << p[k];
    trans[i] = o ^ mask;
  }
  int inv = 0;
  for (int a = 0; a < 3; ++a)
    for (int b = a + 1; b < 3; ++b) inv += p[a] > p[b];
  int flips = ((mask >> 0) & 1) + ((mask >> 1) & 1) + ((mask >> 2) & 1);
  *reflect = ((inv + flips) & 1) != 0;
}

inline int dmc_apply(const int trans[8], int code) {
  int c = 0;
  for (int i = 0; i < 8; ++i)
    if ((code >> trans[i]) & 1) c |= 1 << i;
  return c;
}

inline void dmc_build_table(DmcProc table[256]) {
  for (int idx = 0; idx < 256; ++idx) {
    int best = 256;
    for (int m = 0; m < 8; ++m)
      for (int p = 0; p < 6; ++p) {
        int tr[8];
        bool refl;
        dmc_symmetry(p, m, tr, &refl);
        int c = dmc_apply(tr, idx);
        if (c < best) best = c;
      }
    bool done = false;
    for (int m = 0; m < 8 && !done; ++m)
      for (int p = 0; p < 6 && !done; ++p) {
        int tr[8];
        bool refl;
        dmc_symmetry(p, m, tr, &refl);
        if (dmc_apply(tr, idx) == best) {
          for (int i = 0; i < 8; ++i) table[idx].trans[i] = tr[i];
          table[idx].flip = refl;
          table[idx].code = best;
          done = true;
        }
      }
  }
}

// Dual-cell edge e joins corners (c0, c0 | 1 << axis) with axis = e / 4 and
// the two other corner bits taken from e % 4 (lower axis first).
inline void dmc_edge_corners(int e, int* a, int* b) {
  const int axis = e >> 2, k = e & 3;
  int o0 = axis == 0 ? 1 : 0;
  int o1 = axis == 2 ? 1 : 2;
  int c0 = ((k & 1) << o0) | (((k >> 1) & 1) << o1);
  *a = c0;
  *b = c0 | (1 << axis);
}

struct DmcCase {
  int code;
  const char* tris;  // hex edge indices, three per triangle
};

static const DmcCase kDmcCases[] = {
    {0x01, "048"},
    {0x03, "489549"},
    {0x06, "09449aa95a51"},
    {0x07, "89a1a9519"},
    {0x0f, "89a9ba"},
    {0x16, "0841a55a99a22a6"},
    {0x17, "1a55a929a2a6"},
    {0x18, "15b286"},
    {0x19, "14616bb62b25520"},
    {0x1b, "29669b6b1146"},
    {0x1e, "08429669aa9b"},
    {0x1f, "29669aa9b"},
    {0x3c, "458859a6bb67"},
    {0x3d, "67aa7b059"},
    {0x3f, "67aa7b"},
    {0x69, "05914a26837b"},
    {0x6b, "14818bb8778236a"},
    {0x6f, "26837b"},
    {0x7e, "08437b"},
    {0x7f, "37b"},
};
static const int kNumDmcCases = sizeof(kDmcCases) / sizeof(kDmcCases[0]);

inline int dmc_hex(char c) { return c <= '9' ? c - '0' : c - 'a' + 10; }

// Triangles of canonical code `code` as edge-index triples; returns the count.
inline int dmc_case_tris(int code, int out[][3]) {
  for (int k = 0; k < kNumDmcCases; ++k) {
    if (kDmcCases[k].code != code) continue;
    const char* s = kDmcCases[k].tris;
    int n = (int)std::strlen(s) / 3;
    for (int t = 0; t < n; ++t)
      for (int j = 0; j < 3; ++j) out[t][j] = dmc_hex(s[3 * t + j]);
    return n;
  }
  return 0;
}

}  // namespace pio

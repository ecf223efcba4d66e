// Dual-marching-cubes tables of the extraction stage.
//
// Canonicalisation (the reference's table[256], include/visitorextract.h:35-293):
// a corner-sign code maps to the smallest code of its orbit under the 48 cube
// symmetries; the symmetry used is the first reaching that minimum when
// symmetries are enumerated xor-mask-major (mask 0..7) and, per mask, over
// the axis permutations in kAxisPerms order; `flip` marks orientation-
// reversing symmetries.  This rule regenerates the reference table exactly
// (checked by a CPU test against a digest of it).
//
// Triangles per canonical code (src/visitorextract.cpp:95-199): data that must
// be identical for mesh parity, kept as hex edge-index strings, three edges
// per triangle.  Edge e joins dual-cell corners (c0, c0 | 1 << (e / 4)) with
// the other two corner bits from e % 4, lower axis first
// (dual_edge2vert, include/visitorextract.h:306-311).
#pragma once
#include <cstring>

namespace pisurf {

static const int kAxisPerms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 1, 0}, {2, 0, 1}};

inline void dmc_sym(int pi, int mask, int tr[8], bool* refl) {
  for (int c = 0; c < 8; ++c) {
    int o = 0;
    for (int k = 0; k < 3; ++k) o |= ((c >> k) & 1) << kAxisPerms[pi][k];
    tr[c] = o ^ mask;
  }
  int inv = 0;
  for (int a = 0; a < 3; ++a)
    for (int b = a + 1; b < 3; ++b) inv += kAxisPerms[pi][a] > kAxisPerms[pi][b];
  *refl = ((inv + __builtin_popcount(mask)) & 1) != 0;
}

inline int dmc_permute(const int tr[8], int code) {
  int r = 0;
  for (int c = 0; c < 8; ++c) r |= ((code >> tr[c]) & 1) << c;
  return r;
}

inline void dmc_edge(int e, int* c0, int* c1) {
  const int axis = e >> 2, k = e & 3;
  const int u = axis == 0 ? 1 : 0, v = axis == 2 ? 1 : 2;
  *c0 = ((k & 1) << u) | (((k >> 1) & 1) << v);
  *c1 = *c0 | (1 << axis);
}

struct DmcCaseRow {
  int code;
  const char* edges;
};

static const DmcCaseRow kCaseRows[] = {
    {0x01, "048"},          {0x03, "489549"},          {0x06, "09449aa95a51"},    {0x07, "89a1a9519"},
    {0x0f, "89a9ba"},       {0x16, "0841a55a99a22a6"}, {0x17, "1a55a929a2a6"},    {0x18, "15b286"},
    {0x19, "14616bb62b25520"}, {0x1b, "29669b6b1146"},  {0x1e, "08429669aa9b"},    {0x1f, "29669aa9b"},
    {0x3c, "458859a6bb67"}, {0x3d, "67aa7b059"},       {0x3f, "67aa7b"},          {0x69, "05914a26837b"},
    {0x6b, "14818bb8778236a"}, {0x6f, "26837b"},       {0x7e, "08437b"},          {0x7f, "37b"},
};

struct DmcTables {
  int trans[256][8];
  int flip[256];
  int code[256];
  int ntri[256];       // triangles of canonical code
  int tri[256][15];    // edge triples of canonical code
};

inline void dmc_build(DmcTables* t) {
  std::memset(t, 0, sizeof(*t));
  for (int idx = 0; idx < 256; ++idx) {
    int best = 1 << 30;
    for (int m = 0; m < 8; ++m)
      for (int p = 0; p < 6; ++p) {
        int tr[8];
        bool rf;
        dmc_sym(p, m, tr, &rf);
        int c = dmc_permute(tr, idx);
        best = c < best ? c : best;
      }
    bool set = false;
    for (int m = 0; m < 8 && !set; ++m)
      for (int p = 0; p < 6 && !set; ++p) {
        int tr[8];
        bool rf;
        dmc_sym(p, m, tr, &rf);
        if (dmc_permute(tr, idx) != best) continue;
        for (int c = 0; c < 8; ++c) t->trans[idx][c] = tr[c];
        t->flip[idx] = rf ? 1 : 0;
        t->code[idx] = best;
        set = true;
      }
  }
  for (const DmcCaseRow& r : kCaseRows) {
    int n = (int)std::strlen(r.edges) / 3;
    t->ntri[r.code] = n;
    for (int i = 0; i < 3 * n; ++i) {
      char ch = r.edges[i];
      t->tri[r.code][i] = ch <= '9' ? ch - '0' : ch - 'a' + 10;
    }
  }
}

}  // namespace pisurf

// newick.cpp -- the .tree text of the reference from a join list.
//
// TreeNode::buildTreeOutput (TreeNode.cpp:61-81) writes a leaf as
// name + length and an internal node as "(\n" left ",\n" right ")\n" + length,
// the length being ":" followed by the double with setprecision(4),
// showpoint and setw(8) (empty for the root, whose length stays DBL_MAX);
// SpeciesBlock.cpp:1328-1338 appends ";\n".  The same iostream manipulators
// are used here so the text is identical.
#include <cfloat>
#include <cstring>
#include <iomanip>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/nwgpu.h"

extern "C" int64_t nwg_newick(const nwg_join* joins, int n, const char* const* names, char* out, int64_t cap) {
  if (n < 1 || (n > 1 && !joins) || !names) return -NWG_ERR_INVALID;
  const int nn = 2 * n - 1;
  std::vector<double> length((size_t)nn, DBL_MAX);
  std::vector<int> left((size_t)nn, -1), right((size_t)nn, -1);
  for (int k = 0; k + 1 < n; ++k) {
    const nwg_join& J = joins[k];
    if (J.node != n + k || J.i < 0 || J.j < 0 || J.i >= J.node || J.j >= J.node) return -NWG_ERR_INVALID;
    left[(size_t)J.node] = J.i;
    right[(size_t)J.node] = J.j;
    length[(size_t)J.i] = J.len_i;
    length[(size_t)J.j] = J.len_j;
  }
  std::ostringstream s;
  auto len_text = [&](int v) {
    if (length[(size_t)v] == DBL_MAX) return std::string();
    std::ostringstream t;
    t << ":" << std::setprecision(4) << std::showpoint << std::setw(8) << length[(size_t)v];
    return t.str();
  };
  // iterative pre/in/post-order walk from the root (node nn-1)
  struct Frame { int v; int state; };
  std::vector<Frame> st;
  st.push_back({nn - 1, 0});
  while (!st.empty()) {
    Frame& f = st.back();
    const int v = f.v;
    if (left[(size_t)v] < 0) {
      s << names[v] << len_text(v);
      st.pop_back();
      continue;
    }
    if (f.state == 0) {
      s << "(\n";
      f.state = 1;
      st.push_back({left[(size_t)v], 0});
    } else if (f.state == 1) {
      s << ",\n";
      f.state = 2;
      st.push_back({right[(size_t)v], 0});
    } else {
      s << ")\n" << len_text(v);
      st.pop_back();
    }
  }
  s << ";\n";
  const std::string text = s.str();
  if (out && cap > 0) {
    const int64_t m = (int64_t)text.size() < cap - 1 ? (int64_t)text.size() : cap - 1;
    std::memcpy(out, text.data(), (size_t)m);
    out[m] = 0;
  }
  return (int64_t)text.size();
}

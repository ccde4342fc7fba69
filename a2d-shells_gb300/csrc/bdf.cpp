// Nastran BDF mesh input: the card subset, field layout and renumbering of
// TACSMeshLoader::scanBDFFile (src/io/TACSMeshLoader.cpp:569-1098), so a
// file gives the same node coordinates, element connectivity, components and
// Dirichlet entries as the reference's loader.
//
//   * Bulk data starts after the last "BEGIN BULK" line (the whole file when
//     there is none) and ends at "END BULK" / "ENDDATA"; '$' lines are
//     comments; an empty line inside the bulk data is an error (the
//     reference aborts on it).
//   * GRID: small fixed fields (node 8-16, x 24-32, y 32-40, z 40-48) or
//     comma-separated free fields; GRID*: large fields (node 8-24, x 40-56,
//     y 56-72, z on the next line at 8-24).
//   * SPC: node 16-24, DOF digits 24-32, value 32-40; SPC*: node 24-40,
//     digits 40-56, value 56-72.  Digit d fixes variable d - 1 (1..8).  One
//     node per card.
//   * Element cards, first matching prefix of CBAR CQUADR CQUAD4 CQUAD8
//     CQUAD9 CQUAD CHEXA27 CHEXA CTRIA3 CTETRA ('*' after the name: 16-wide
//     fields): element number and component at fields 1-2, then node
//     numbers; blank fields are skipped, a field reading <= 0 (or cut short
//     by the end of the line) ends the list, and a following line that
//     starts with ' ' or '*' continues it (from column 8).  Node order is converted to the tensor-product order of
//     the shell elements for CQUAD4/CQUADR, CQUAD9/CQUAD and CHEXA
//     (TACSMeshLoader.cpp:932-956).
//   * Reals accept the Nastran short exponent forms (1.5-3, 2.+4) and D
//     exponents (bdf_atof, TACSMeshLoader.cpp:176-217).
//   * Nodes are numbered by sorted file node number and elements by sorted
//     file element number; connectivity and SPC nodes are mapped to that
//     numbering (an unknown node number is an error).
//   * "$       Shell" comment lines name the components in order (the
//     first word from column 41).
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cctype>
#include <new>
#include <string>
#include <vector>

#include "a2ds.h"
#include "a2ds_internal.h"

namespace a2ds {

struct BdfMesh {
  int num_nodes = 0, num_elements = 0, num_components = 0, num_bcs = 0;
  std::vector<double> X;                            // num_nodes x 3, sorted node order
  std::vector<int> elem_ptr, elem_conn, elem_comp;  // sorted element order
  std::vector<int> bc_nodes, bc_ptr, bc_vars;
  std::vector<double> bc_vals;
  std::vector<std::string> comp_elems, comp_descript;
};

namespace {

const char *const kElemTypes[] = {"CBAR",    "CQUADR", "CQUAD4", "CQUAD8", "CQUAD9",
                                  "CQUAD",   "CHEXA27", "CHEXA", "CTRIA3", "CTETRA"};
const int kElemLimits[][2] = {{2, 2}, {4, 4},   {4, 4}, {8, 8}, {9, 9},
                              {9, 9}, {27, 27}, {8, 8}, {3, 3}, {4, 10}};
constexpr int kNumElemTypes = 10;
constexpr size_t kLineMax = 80;

// The file split into lines ('\n' separated, at most 80 characters kept).
struct Lines {
  std::vector<std::string> v;
  explicit Lines(const std::string &buf) {
    size_t p = 0;
    while (p < buf.size()) {
      size_t e = buf.find('\n', p);
      if (e == std::string::npos) e = buf.size();
      v.push_back(buf.substr(p, std::min(e - p, kLineMax)));
      p = e + 1;
    }
  }
};

// Characters [a, a + w) of a line, empty past its end.
std::string field(const std::string &line, size_t a, size_t w) {
  if (a >= line.size()) return std::string();
  return line.substr(a, w);
}

int to_int(const std::string &s) { return atoi(s.c_str()); }

// A Nastran real: E/e exponents as is, D/d exponents as E, otherwise a sign
// after the first character (a leading minus excepted) starts the exponent.
double bdf_real(const std::string &in) {
  std::string s = in;
  for (size_t i = 0; i < s.size(); i++) {
    if (s[i] == 'e' || s[i] == 'E') return atof(s.c_str());
    if (s[i] == 'd' || s[i] == 'D') {
      s[i] = 'e';
      return atof(s.c_str());
    }
  }
  size_t i = 0;
  while (i < s.size() && s[i] == ' ') i++;
  if (i == s.size()) return 0.0;
  std::string t;
  if (s[i] == '-') t += s[i++];
  for (; i < s.size(); i++) {
    if (s[i] == '-' || s[i] == '+') t += 'e';
    t += s[i];
  }
  return atof(t.c_str());
}

bool blank(const std::string &s) {
  for (char c : s)
    if (!isspace((unsigned char)c)) return false;
  return true;
}

// Element card at line k: number, component and up to max_nodes node
// numbers over the continuation lines; k is left at the last line used.
// Returns false when the element or component number is not positive.
bool parse_element(const Lines &L, size_t &k, size_t width, int max_nodes, int &elem, int &comp,
                   std::vector<int> &nodes) {
  nodes.clear();
  std::string line = L.v[k];
  size_t at = 8;
  elem = to_int(field(line, at, width));
  at += width;
  if (elem <= 0) return false;
  comp = to_int(field(line, at, width));
  at += width;
  if (comp <= 0) return false;
  while ((int)nodes.size() < max_nodes) {
    for (; (int)nodes.size() < max_nodes && at < line.size(); at += width) {
      // blank only when the whole field is present and white (a field cut
      // short by the end of the line, e.g. a trailing "\r", reads as 0 and
      // ends the list, as in the reference)
      const std::string f = field(line, at, width);
      if (f.size() == width && blank(f)) continue;
      const int v = to_int(f);
      if (v <= 0) return true;  // end of the node list
      nodes.push_back(v);
    }
    if ((int)nodes.size() < max_nodes) {
      if (k + 1 >= L.v.size()) return true;
      const std::string &next = L.v[k + 1];
      if (next.empty() || !(next[0] == '*' || next[0] == ' ')) return true;
      line = next;
      k++;
      at = 8;
    }
  }
  return true;
}

}  // namespace

// Parse `buf` into m; returns 0 or an A2DS_ERR_* code with the message set.
int bdf_parse(const std::string &buf, BdfMesh &m) {
  const Lines L(buf);
  const size_t nlines = L.v.size();
  size_t k0 = 0;
  // the reader looks at every line but the last for BEGIN BULK
  for (size_t k = 0; k + 1 < nlines; k++)
    if (L.v[k].compare(0, 10, "BEGIN BULK") == 0) k0 = k + 1;

  std::vector<int> node_num, elem_num, elem_comp, conn_ptr(1, 0), conn;
  std::vector<double> Xf;
  std::vector<int> bc_node_num;
  std::vector<std::string> descripts;
  m.bc_ptr.assign(1, 0);
  m.bc_vars.clear();
  m.bc_vals.clear();
  std::vector<int> nodes;
  for (size_t k = k0; k < nlines; k++) {
    const std::string &line = L.v[k];
    if (line.empty())
      return fail(A2DS_ERR_ARG, "BDF: empty line " + std::to_string(k + 1) + " in the bulk data");
    if (line.compare(0, 13, "$       Shell") == 0) {
      std::string w = field(line, 41, 32);
      char word[33] = {0};
      if (sscanf(w.c_str(), "%32s", word) != 1) word[0] = '\0';
      descripts.push_back(word);
    }
    if (line[0] == '$') continue;
    if (line.compare(0, 8, "END BULK") == 0 || line.compare(0, 7, "ENDDATA") == 0) break;
    if (line.compare(0, 5, "GRID*") == 0) {
      if (k + 1 >= nlines || L.v[k + 1].empty())
        return fail(A2DS_ERR_ARG, "BDF: GRID* without its second line at line " +
                                      std::to_string(k + 1));
      const std::string &l2 = L.v[k + 1];
      node_num.push_back(to_int(field(line, 8, 16)) - 1);
      Xf.push_back(bdf_real(field(line, 40, 16)));
      Xf.push_back(bdf_real(field(line, 56, 16)));
      Xf.push_back(bdf_real(field(l2, 8, 16)));
      k++;
    } else if (line.compare(0, 4, "GRID") == 0) {
      std::string f[5];
      if (line.find(',') != std::string::npos) {  // free field
        size_t end = 8;
        for (int i = 0; i < 5; i++) {
          const size_t start = end;
          while (end < line.size() && line[end] != ',') end++;
          f[i] = start < line.size() ? line.substr(start, end - start) : std::string();
          end++;
        }
      } else {
        f[0] = field(line, 8, 8);
        f[2] = field(line, 24, 8);
        f[3] = field(line, 32, 8);
        f[4] = field(line, 40, 8);
      }
      node_num.push_back(to_int(f[0]) - 1);
      Xf.push_back(bdf_real(f[2]));
      Xf.push_back(bdf_real(f[3]));
      Xf.push_back(bdf_real(f[4]));
    } else if (line.compare(0, 3, "SPC") == 0) {
      const bool wide = line.compare(0, 4, "SPC*") == 0;
      const size_t w = wide ? 16 : 8, at = wide ? 24 : 16;
      bc_node_num.push_back(to_int(field(line, at, w)) - 1);
      const double val = bdf_real(field(line, at + 2 * w, w));
      const std::string dofs = field(line, at + w, w);
      for (char c : dofs)
        if (c >= '1' && c <= '8') {
          m.bc_vars.push_back(c - '1');
          m.bc_vals.push_back(val);
        }
      m.bc_ptr.push_back((int)m.bc_vars.size());
    } else {
      int index = -1;
      size_t width = 8;
      for (int t = 0; t < kNumElemTypes; t++) {
        const size_t len = strlen(kElemTypes[t]);
        if (line.compare(0, len, kElemTypes[t]) == 0) {
          index = t;
          if (line.size() > len && line[len] == '*') width = 16;
          break;
        }
      }
      if (index < 0) continue;  // not a card this loader reads
      int e = 0, c = 0;
      const size_t kfirst = k;
      if (!parse_element(L, k, width, kElemLimits[index][1], e, c, nodes))
        return fail(A2DS_ERR_ARG, "BDF: element or component number not positive at line " +
                                      std::to_string(kfirst + 1));
      const int nc = (int)nodes.size();
      if (nc < kElemLimits[index][0])
        return fail(A2DS_ERR_ARG, std::string("BDF: too few nodes for element ") +
                                      kElemTypes[index] + " at line " + std::to_string(kfirst + 1));
      static const int q4[4] = {0, 1, 3, 2};
      static const int q9[9] = {0, 4, 1, 7, 8, 5, 3, 6, 2};
      static const int h8[8] = {0, 1, 3, 2, 4, 5, 7, 6};
      const std::string &first = L.v[kfirst];
      const int *perm = nullptr;
      int np = nc;
      if (first.compare(0, 6, "CQUAD4") == 0 || first.compare(0, 6, "CQUADR") == 0) {
        perm = q4;
        np = 4;
      } else if (first.compare(0, 6, "CQUAD9") == 0 || first.compare(0, 5, "CQUAD") == 0) {
        if (nc < 9)
          return fail(A2DS_ERR_ARG, "BDF: CQUAD card with fewer than 9 nodes at line " +
                                        std::to_string(kfirst + 1));
        perm = q9;
        np = 9;
      } else if (first.compare(0, 5, "CHEXA") == 0) {
        if (nc != 8)
          return fail(A2DS_ERR_ARG, "BDF: only 8-node CHEXA cards are supported (line " +
                                        std::to_string(kfirst + 1) + ")");
        perm = h8;
        np = 8;
      }
      for (int a = 0; a < nc; a++) conn.push_back((perm && a < np ? nodes[perm[a]] : nodes[a]) - 1);
      conn_ptr.push_back((int)conn.size());
      elem_num.push_back(e - 1);
      elem_comp.push_back(c - 1);
      if (c > (int)m.comp_elems.size()) m.comp_elems.resize(c);
      if (m.comp_elems[c - 1].empty())
        m.comp_elems[c - 1] = (first.compare(0, 6, "CTETRA") == 0 && nc == 10)
                                  ? std::string("CTETRA10")
                                  : std::string(kElemTypes[index]);
    }
  }

  // renumber: nodes by file node number, elements by file element number
  const int nn = (int)node_num.size(), ne = (int)elem_num.size();
  std::vector<int> nord(nn), eord(ne);
  for (int i = 0; i < nn; i++) nord[i] = i;
  for (int i = 0; i < ne; i++) eord[i] = i;
  std::stable_sort(nord.begin(), nord.end(),
                   [&](int a, int b) { return node_num[a] < node_num[b]; });
  std::stable_sort(eord.begin(), eord.end(),
                   [&](int a, int b) { return elem_num[a] < elem_num[b]; });
  std::vector<int> sorted_num(nn);
  for (int i = 0; i < nn; i++) sorted_num[i] = node_num[nord[i]];
  auto lookup = [&](int num) {
    auto it = std::lower_bound(sorted_num.begin(), sorted_num.end(), num);
    return (it != sorted_num.end() && *it == num) ? (int)(it - sorted_num.begin()) : -1;
  };
  m.num_nodes = nn;
  m.num_elements = ne;
  m.num_components = (int)m.comp_elems.size();
  m.X.resize((size_t)nn * 3);
  for (int i = 0; i < nn; i++)
    for (int d = 0; d < 3; d++) m.X[(size_t)i * 3 + d] = Xf[(size_t)nord[i] * 3 + d];
  m.elem_ptr.assign(1, 0);
  m.elem_conn.clear();
  m.elem_comp.resize(ne);
  for (int k = 0; k < ne; k++) {
    const int e = eord[k];
    for (int j = conn_ptr[e]; j < conn_ptr[e + 1]; j++) {
      const int v = lookup(conn[j]);
      if (v < 0)
        return fail(A2DS_ERR_ARG, "BDF: element " + std::to_string(elem_num[e] + 1) +
                                      " uses undefined node " + std::to_string(conn[j] + 1));
      m.elem_conn.push_back(v);
    }
    m.elem_comp[k] = elem_comp[e];
    m.elem_ptr.push_back((int)m.elem_conn.size());
  }
  m.num_bcs = (int)bc_node_num.size();
  m.bc_nodes.resize(m.num_bcs);
  for (int b = 0; b < m.num_bcs; b++) {
    const int v = lookup(bc_node_num[b]);
    if (v < 0)
      return fail(A2DS_ERR_ARG, "BDF: SPC on undefined node " + std::to_string(bc_node_num[b] + 1));
    m.bc_nodes[b] = v;
  }
  m.comp_descript.assign(m.num_components, std::string());
  for (size_t d = 0; d < descripts.size() && (int)d < m.num_components; d++)
    m.comp_descript[d] = descripts[d];
  return 0;
}

}  // namespace a2ds

using a2ds::BdfMesh;
struct a2ds_bdf_s {
  BdfMesh m;
};

#define BDF_GUARD_BEGIN try {
#define BDF_GUARD_END                                              \
  }                                                                \
  catch (const std::bad_alloc &) {                                 \
    return a2ds::fail(A2DS_ERR_NOMEM, "host allocation failed");   \
  }                                                                \
  catch (...) {                                                    \
    return a2ds::fail(A2DS_ERR_STATE, "unexpected host exception"); \
  }

extern "C" {

int a2ds_bdf_scan(const char *file_name, a2ds_bdf *out) {
  BDF_GUARD_BEGIN
  if (!out || !file_name) return a2ds::fail(A2DS_ERR_ARG, "file_name and out are required");
  *out = nullptr;
  FILE *fp = fopen(file_name, "rb");
  if (!fp) return a2ds::fail(A2DS_ERR_ARG, std::string("BDF: cannot open ") + file_name);
  std::string buf;
  char chunk[1 << 16];
  size_t got;
  while ((got = fread(chunk, 1, sizeof(chunk), fp)) > 0) buf.append(chunk, got);
  fclose(fp);
  a2ds_bdf h = new a2ds_bdf_s();
  const int rc = a2ds::bdf_parse(buf, h->m);
  if (rc) {
    delete h;
    return rc;
  }
  *out = h;
  return 0;
  BDF_GUARD_END
}

int a2ds_bdf_destroy(a2ds_bdf bdf) {
  delete bdf;
  return 0;
}

int a2ds_bdf_get_sizes(a2ds_bdf bdf, int *num_nodes, int *num_elements, int *conn_size,
                       int *num_bcs, int *bc_vars_size, int *num_components) {
  if (!bdf) return a2ds::fail(A2DS_ERR_ARG, "null BDF handle");
  const BdfMesh &m = bdf->m;
  if (num_nodes) *num_nodes = m.num_nodes;
  if (num_elements) *num_elements = m.num_elements;
  if (conn_size) *conn_size = (int)m.elem_conn.size();
  if (num_bcs) *num_bcs = m.num_bcs;
  if (bc_vars_size) *bc_vars_size = (int)m.bc_vars.size();
  if (num_components) *num_components = m.num_components;
  return 0;
}

int a2ds_bdf_get_connectivity(a2ds_bdf bdf, int *elem_node_ptr, int *elem_node_conn,
                              int *elem_component, double *Xpts) {
  if (!bdf) return a2ds::fail(A2DS_ERR_ARG, "null BDF handle");
  const BdfMesh &m = bdf->m;
  if (elem_node_ptr) std::copy(m.elem_ptr.begin(), m.elem_ptr.end(), elem_node_ptr);
  if (elem_node_conn) std::copy(m.elem_conn.begin(), m.elem_conn.end(), elem_node_conn);
  if (elem_component) std::copy(m.elem_comp.begin(), m.elem_comp.end(), elem_component);
  if (Xpts) std::copy(m.X.begin(), m.X.end(), Xpts);
  return 0;
}

int a2ds_bdf_get_bcs(a2ds_bdf bdf, int *bc_nodes, int *bc_vars, int *bc_ptr, double *bc_vals) {
  if (!bdf) return a2ds::fail(A2DS_ERR_ARG, "null BDF handle");
  const BdfMesh &m = bdf->m;
  if (bc_nodes) std::copy(m.bc_nodes.begin(), m.bc_nodes.end(), bc_nodes);
  if (bc_vars) std::copy(m.bc_vars.begin(), m.bc_vars.end(), bc_vars);
  if (bc_ptr) std::copy(m.bc_ptr.begin(), m.bc_ptr.end(), bc_ptr);
  if (bc_vals) std::copy(m.bc_vals.begin(), m.bc_vals.end(), bc_vals);
  return 0;
}

static int copy_name(const std::string &s, char *out, int len) {
  if (!out || len <= 0) return a2ds::fail(A2DS_ERR_ARG, "output buffer required");
  const size_t n = std::min(s.size(), (size_t)len - 1);
  memcpy(out, s.data(), n);
  out[n] = '\0';
  return 0;
}

int a2ds_bdf_get_element_descript(a2ds_bdf bdf, int comp, char *name, int len) {
  if (!bdf) return a2ds::fail(A2DS_ERR_ARG, "null BDF handle");
  if (comp < 0 || comp >= bdf->m.num_components)
    return a2ds::fail(A2DS_ERR_ARG, "component out of range");
  return copy_name(bdf->m.comp_elems[comp], name, len);
}

int a2ds_bdf_get_component_descript(a2ds_bdf bdf, int comp, char *descript, int len) {
  if (!bdf) return a2ds::fail(A2DS_ERR_ARG, "null BDF handle");
  if (comp < 0 || comp >= bdf->m.num_components)
    return a2ds::fail(A2DS_ERR_ARG, "component out of range");
  return copy_name(bdf->m.comp_descript[comp], descript, len);
}

}  // extern "C"

// .f5 output: the binary layout TACSToFH5::writeToFile writes through
// TACSFH5File (src/io/TACSToFH5.cpp:126-358, src/io/TACSFH5.cpp:64-210) for
// one process, for every output class of a shell mesh (TACS_OUTPUT_*).
//
// File = header + zones, native byte order.
//   header: int num_components; per component: int length (with the NUL),
//           the name and its NUL ("Component k" when no name is given).
//   zone:   int {type (0 int, 2 float), dim1, dim2, len(zone)+1,
//           len(vars)+1}, zone name + NUL, variable names + NUL, then
//           dim1 x dim2 values (4-byte int or float).
// Zones, in order: with CONNECTIVITY "components" (component of each
// element), "ltypes" (element layout: 8 = Quad4, 9 = Quad9), "ptr"
// (num_elements + 1 offsets), "connectivity"; with NODES and/or
// DISPLACEMENTS and/or LOADS one float zone "continuous data t=<time %.10e>"
// with variables "X,Y,Z", then "u,v,w,rotx,roty,rotz", then
// "fx,fy,fz,mx,my,mz" (the residual at vars without external loads,
// assembleRes(F, 0.0), which needs an initialized mesh), one row per node;
// with STRAINS, STRESSES and/or EXTRAS one float zone "element data
// t=<time>" with one row per element node point (TACSShellElement::
// getOutputData, src/elements/shell/TACSShellElement.h:1404-1515).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "a2ds.h"
#include "a2ds_internal.h"
#include "runtime.h"

namespace {

constexpr int kF5Int = 0, kF5Float = 2;
constexpr int kLayoutQuad = 8, kLayoutQuadQuadratic = 9;

void put_int(std::vector<char> &b, int v) {
  const char *p = reinterpret_cast<const char *>(&v);
  b.insert(b.end(), p, p + sizeof(int));
}

void put_str(std::vector<char> &b, const std::string &s) {
  b.insert(b.end(), s.begin(), s.end());
  b.push_back('\0');
}

template <typename T>
void put_zone(std::vector<char> &b, int type, const std::string &zone, const std::string &vars,
              int dim1, int dim2, const T *data) {
  put_int(b, type);
  put_int(b, dim1);
  put_int(b, dim2);
  put_int(b, (int)zone.size() + 1);
  put_int(b, (int)vars.size() + 1);
  put_str(b, zone);
  put_str(b, vars);
  const char *p = reinterpret_cast<const char *>(data);
  b.insert(b.end(), p, p + sizeof(T) * (size_t)dim1 * dim2);
}

// Element output at every element's node points (getOutputData order:
// strains e, stresses C e, extras), element-major; names as
// TACSToFH5::getElementVarNames for TACS_BEAM_OR_SHELL_ELEMENT.
int element_data(a2ds_mesh mesh, int eflags, const double *vars, std::vector<float> &v,
                 std::string &names) {
  using namespace a2ds;
  Mesh &m = mesh->m;
  if (!m.initialized) return fail(A2DS_ERR_STATE, "element output needs an initialized mesh");
  const int ne = m.ne, npe = m.npe;
  int rc;
  const double *dst = nullptr;
  if (vars) {
    if ((rc = m.to_rows(vars, m.d_state))) return rc;
    dst = m.d_state.p;
  }
  DBuf<double> dout;
  if ((rc = dout.alloc((size_t)ne * npe * 18))) return rc;
  if ((rc = m.element_output(dst, dout.p))) return rc;
  std::vector<double> h((size_t)ne * npe * 18);
  A2DS_CUDA_TRY(cudaMemcpyAsync(h.data(), dout.p, h.size() * sizeof(double),
                                cudaMemcpyDeviceToHost, m.stream));
  A2DS_CUDA_TRY(cudaStreamSynchronize(m.stream));
  const bool st = eflags & A2DS_F5_STRAINS, ss = eflags & A2DS_F5_STRESSES,
             ex = eflags & A2DS_F5_EXTRAS;
  static const char *kStrain = "ex0,ey0,exy0,ex1,ey1,exy1,eyz0,exz0,erot";
  static const char *kStress = "sx0,sy0,sxy0,sx1,sy1,sxy1,syz0,sxz0,srot";
  static const char *kExtra =
      "failure0,failure1,failure2,failure3,failure4,failure5,dv1,dv2,dv3,dv4,dv5,dv6,dv7";
  names.clear();
  for (const char *part : {st ? kStrain : nullptr, ss ? kStress : nullptr, ex ? kExtra : nullptr})
    if (part) names += (names.empty() ? "" : ",") + std::string(part);
  const int nvals = (st ? 9 : 0) + (ss ? 9 : 0) + (ex ? 13 : 0);
  v.assign((size_t)ne * npe * nvals, 0.0f);
  // plane-stress tangent of the isotropic material (evalTangentStiffness2D)
  const double D = m.E / (1.0 - m.nu * m.nu), G = 0.5 * m.E / (1.0 + m.nu);
  const double C[6] = {D, m.nu * D, 0.0, D, 0.0, G};
  for (int e = 0; e < ne; e++) {
    const double t = m.tvals[m.tgroup.empty() ? 0 : m.tgroup[e]];
    for (int q = 0; q < npe; q++) {
      const double *o = &h[((size_t)e * npe + q) * 18];
      float *w = &v[((size_t)e * npe + q) * nvals];
      if (st)
        for (int i = 0; i < 9; i++) *w++ = (float)o[i];
      if (ss)
        for (int i = 0; i < 9; i++) *w++ = (float)o[9 + i];
      if (ex) {
        // failure0: KS (weight 100) of the von Mises failure of the top and
        // bottom surfaces (TACSIsoShellConstitutive::evalFailure, tOffset 0)
        double fail2[2];
        for (int side = 0; side < 2; side++) {
          const double z = (side == 0 ? 0.5 : -0.5) * t;  // surface offset
          const double es[3] = {o[0] + z * o[3], o[1] + z * o[4], o[2] + z * o[5]};
          const double sv[3] = {C[0] * es[0] + C[1] * es[1] + C[2] * es[2],
                                C[1] * es[0] + C[3] * es[1] + C[4] * es[2],
                                C[2] * es[0] + C[4] * es[1] + C[5] * es[2]};
          fail2[side] =
              sqrt(sv[0] * sv[0] + sv[1] * sv[1] - sv[0] * sv[1] + 3.0 * sv[2] * sv[2]) / m.ys;
        }
        const double ksw = 100.0;
        const double mx = fail2[0] > fail2[1] ? fail2[0] : fail2[1];
        const double ks = mx + log(exp(ksw * (fail2[0] - mx)) + exp(ksw * (fail2[1] - mx))) / ksw;
        *w++ = (float)ks;
        for (int i = 1; i < 6; i++) *w++ = 0.0f;  // failure1-5
        *w++ = (float)t;                           // dv1: the thickness
        for (int i = 1; i < 7; i++) *w++ = 0.0f;  // dv2-7
      }
    }
  }
  return 0;
}

}  // namespace

extern "C" int a2ds_write_f5(a2ds_mesh mesh, const char *file_name, int write_flag,
                             int num_components, const char *const *component_names,
                             const int *elem_component, const double *vars, double time) {
  try {
    using a2ds::fail;
    if (!mesh || !file_name) return fail(A2DS_ERR_ARG, "mesh and file_name are required");
    const int allowed = A2DS_F5_CONNECTIVITY | A2DS_F5_NODES | A2DS_F5_DISPLACEMENTS |
                        A2DS_F5_STRAINS | A2DS_F5_STRESSES | A2DS_F5_EXTRAS | A2DS_F5_LOADS;
    if (write_flag & ~allowed) return fail(A2DS_ERR_ARG, "write_flag: unknown output class");
    if ((write_flag & A2DS_F5_EXTRAS) && !(mesh->m.ys > 0.0))
      return fail(A2DS_ERR_STATE, "extras (failure values) need a2ds_mesh_set_yield_stress");
    const a2ds::Mesh &m = mesh->m;
    const int ne = m.ne, nn = m.nn, npe = m.npe;
    int maxc = 0;
    if (elem_component)
      for (int e = 0; e < ne; e++) {
        if (elem_component[e] < 0) return fail(A2DS_ERR_ARG, "negative component number");
        maxc = std::max(maxc, elem_component[e]);
      }
    // TACSAssembler::getNumComponents: largest component number + 1 (the
    // caller's names cover its own num_components entries only)
    const int given = component_names ? std::max(num_components, 0) : 0;
    if (num_components < maxc + 1) num_components = maxc + 1;
    std::vector<char> b;
    put_int(b, num_components);
    for (int k = 0; k < num_components; k++) {
      std::string name = (k < given && component_names[k])
                             ? std::string(component_names[k])
                             : "Component " + std::to_string(k);
      put_int(b, (int)name.size() + 1);
      put_str(b, name);
    }
    if (write_flag & A2DS_F5_CONNECTIVITY) {
      std::vector<int> comp(ne, 0), lt(ne, npe == 4 ? kLayoutQuad : kLayoutQuadQuadratic),
          ptr(ne + 1);
      if (elem_component) std::copy(elem_component, elem_component + ne, comp.begin());
      for (int e = 0; e <= ne; e++) ptr[e] = npe * e;
      put_zone(b, kF5Int, "components", "components", ne, 1, comp.data());
      put_zone(b, kF5Int, "ltypes", "ltypes", ne, 1, lt.data());
      put_zone(b, kF5Int, "ptr", "ptr", ne + 1, 1, ptr.data());
      put_zone(b, kF5Int, "connectivity", "connectivity", ne * npe, 1, m.conn.data());
    }
    const bool nodes = write_flag & A2DS_F5_NODES, disp = write_flag & A2DS_F5_DISPLACEMENTS;
    const bool loads = write_flag & A2DS_F5_LOADS;
    std::vector<double> res;
    if (loads) {  // assembleRes(F, 0.0) at vars: internal forces, BC rows as the reference
      res.resize((size_t)nn * 6);
      std::vector<double> zero;
      if (!vars) zero.assign((size_t)nn * 6, 0.0);
      const int rc = a2ds_assemble_res(mesh, vars ? vars : zero.data(), res.data());
      if (rc) return rc;
    }
    if (nodes || disp || loads) {
      std::string names = nodes ? "X,Y,Z" : "";
      if (disp) names += std::string(nodes ? "," : "") + "u,v,w,rotx,roty,rotz";
      if (loads) names += std::string(nodes || disp ? "," : "") + "fx,fy,fz,mx,my,mz";
      const int dim2 = (nodes ? 3 : 0) + (disp ? 6 : 0) + (loads ? 6 : 0);
      const int off = nodes ? 3 : 0, loff = off + (disp ? 6 : 0);
      std::vector<float> v((size_t)nn * dim2, 0.0f);
      for (int i = 0; i < nn; i++) {
        if (nodes)
          for (int j = 0; j < 3; j++) v[(size_t)i * dim2 + j] = (float)m.X[(size_t)i * 3 + j];
        if (disp)
          for (int j = 0; j < 6; j++)
            v[(size_t)i * dim2 + off + j] = vars ? (float)vars[(size_t)i * 6 + j] : 0.0f;
        if (loads)
          for (int j = 0; j < 6; j++) v[(size_t)i * dim2 + loff + j] = (float)res[(size_t)i * 6 + j];
      }
      char zone[128];
      snprintf(zone, sizeof(zone), "continuous data t=%.10e", time);
      put_zone(b, kF5Float, zone, names, nn, dim2, v.data());
    }
    const int eflags = write_flag & (A2DS_F5_STRAINS | A2DS_F5_STRESSES | A2DS_F5_EXTRAS);
    if (eflags) {
      std::vector<float> v;
      std::string names;
      int rc = element_data(mesh, eflags, vars, v, names);
      if (rc) return rc;
      char zone[128];
      snprintf(zone, sizeof(zone), "element data t=%.10e", time);
      const int nvals = (int)(v.size() / ((size_t)ne * npe));
      put_zone(b, kF5Float, zone, names, ne * npe, nvals, v.data());
    }
    FILE *fp = fopen(file_name, "wb");
    if (!fp) return fail(A2DS_ERR_ARG, std::string("cannot create ") + file_name);
    const size_t w = fwrite(b.data(), 1, b.size(), fp);
    const int c = fclose(fp);
    if (w != b.size() || c != 0) return fail(A2DS_ERR_STATE, std::string("short write to ") + file_name);
    return 0;
  } catch (const std::bad_alloc &) {
    return a2ds::fail(A2DS_ERR_NOMEM, "host allocation failed");
  } catch (...) {
    return a2ds::fail(A2DS_ERR_STATE, "unexpected host exception");
  }
}

// Mesh input and field output in ModFEM's file formats (host code).
//
//  * jk ("gradmesh") prism meshes, read as mmr_import_mesh_grad does
//    (mmd_prism/mms_prism_input_gradmesh.c:30-420): a 2D triangle mesh
//    extruded in num_el_lay layers; nodes, elements and faces numbered as the
//    reference numbers them, so results map one to one onto its entities;
//  * field dumps (field.dmp) as apr_write_field writes them for std fields
//    (apd_std_lin/aps_std_lin_intf.c:539-680: "nreq nr_sol", the number of
//    DOF entities, then one line per vertex "id value ...", "%.12lg ") and DG
//    fields (apd_dg_prism/aps_dg_prism_intf.c:459-560: "nreq nr_sol", -pdeg
//    once (uniform) or per element, then one line of coefficients per
//    element, values below 1e-15 written as 0).

#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "gbfem_internal.h"

namespace {

struct JkFace {
  int type, bc, el1, el2, side1, nodes[4];
};

struct JkMesh {
  int nno = 0, nel = 0;
  std::vector<double> xyz;
  std::vector<int> el;
  std::vector<JkFace> faces;
};

int read_jk(const char *path, JkMesh &M) {
  FILE *fp = fopen(path, "r");
  GB_CHECK(fp, std::string("cannot open jk file ") + path);
  int mx[4], nn2d = 0, nlay = 0, bbc = 0, tbc = 0, ne2d = 0;
  double zb = 0, zt = 0;
  bool ok = fscanf(fp, "%d %d %d %d", mx, mx + 1, mx + 2, mx + 3) == 4 &&
            fscanf(fp, "%d %lg %lg %d %d %d", &nn2d, &zb, &zt, &nlay, &bbc, &tbc) == 6 && nn2d > 0 && nlay > 0;
  std::vector<double> xy(2 * (size_t)std::max(nn2d, 0));
  for (int i = 0; ok && i < nn2d; i++) ok = fscanf(fp, "%lg %lg", &xy[2 * i], &xy[2 * i + 1]) == 2;
  ok = ok && fscanf(fp, "%d", &ne2d) == 1 && ne2d > 0;
  std::vector<int> tri(3 * (size_t)std::max(ne2d, 0)), nb(3 * (size_t)std::max(ne2d, 0));
  for (int t = 0; ok && t < ne2d; t++) {
    int mat = 0;
    ok = fscanf(fp, "%d", &mat) == 1 && mat > 0;  // triangles only (prisms)
    for (int j = 0; ok && j < 3; j++) ok = fscanf(fp, "%d", &tri[3 * t + j]) == 1 && tri[3 * t + j] >= 1 &&
                                           tri[3 * t + j] <= nn2d;
    for (int j = 0; ok && j < 3; j++) ok = fscanf(fp, "%d", &nb[3 * t + j]) == 1 && nb[3 * t + j] != 0 &&
                                           nb[3 * t + j] <= ne2d;
  }
  fclose(fp);
  GB_CHECK(ok, std::string("malformed or unsupported jk file (triangle layers only) ") + path);
  const double dz = (zt - zb) / nlay;
  M.nno = nn2d * (nlay + 1);
  M.nel = ne2d * nlay;
  M.xyz.assign(3 * (size_t)M.nno, 0.0);
  for (int i = 0; i < nn2d; i++)
    for (int l = 0; l <= nlay; l++) {
      double *p = &M.xyz[3 * ((size_t)i + (size_t)l * nn2d)];
      p[0] = xy[2 * i];
      p[1] = xy[2 * i + 1];
      p[2] = zb + l * dz;
    }
  M.el.assign(6 * (size_t)M.nel, 0);
  for (int t = 0; t < ne2d; t++)
    for (int l = 0; l < nlay; l++) {
      int *e = &M.el[6 * ((size_t)t + (size_t)l * ne2d)];
      for (int j = 0; j < 3; j++) {
        e[j] = tri[3 * t + j] - 1 + l * nn2d;
        e[3 + j] = tri[3 * t + j] - 1 + (l + 1) * nn2d;
      }
    }
  // horizontal faces: id = t + 1 + level * ne2d
  const int nr_hor = ne2d * (nlay + 1);
  M.faces.assign(nr_hor, JkFace());
  for (int l = 0; l <= nlay; l++)
    for (int t = 0; t < ne2d; t++) {
      JkFace &f = M.faces[t + (size_t)l * ne2d];
      const int v0 = tri[3 * t] - 1 + l * nn2d, v1 = tri[3 * t + 1] - 1 + l * nn2d, v2 = tri[3 * t + 2] - 1 + l * nn2d;
      f.type = 3;
      f.nodes[3] = -1;
      if (l == 0) {
        f.bc = bbc; f.el1 = t; f.el2 = -1; f.side1 = 0;
        f.nodes[0] = v0; f.nodes[1] = v2; f.nodes[2] = v1;
      } else {
        f.bc = l == nlay ? tbc : 0;
        f.el1 = t + (l - 1) * ne2d;
        f.el2 = l == nlay ? -1 : t + l * ne2d;
        f.side1 = 1;
        f.nodes[0] = v0; f.nodes[1] = v1; f.nodes[2] = v2;
      }
    }
  // vertical faces in creation order: the first element of a pair creates
  // the column of faces over its edge (quadrilaterals a, b, b', a')
  std::map<std::pair<int, int>, int> made;
  for (int t = 0; t < ne2d; t++)
    for (int j = 0; j < 3; j++) {
      const int g = nb[3 * t + j];
      if (g > 0 && made.count({std::min(t + 1, g), std::max(t + 1, g)})) continue;
      if (g > 0) made[{std::min(t + 1, g), std::max(t + 1, g)}] = 1;
      const int a = tri[3 * t + j] - 1, b = tri[3 * t + (j + 1) % 3] - 1;
      for (int l = 0; l < nlay; l++) {
        JkFace f;
        f.type = 4;
        f.bc = g > 0 ? -1 : -g;
        f.el1 = t + l * ne2d;
        f.el2 = g > 0 ? g - 1 + l * ne2d : -1;
        f.side1 = 2 + j;
        f.nodes[0] = a + l * nn2d;
        f.nodes[1] = b + l * nn2d;
        f.nodes[2] = b + (l + 1) * nn2d;
        f.nodes[3] = a + (l + 1) * nn2d;
        M.faces.push_back(f);
      }
    }
  return 0;
}

}  // namespace

extern "C" {

int gbfem_read_jk(const char *path, int *sizes, double *xyz, int *el_nodes, int *fa_type, int *fa_bc, int *fa_el,
                  int *fa_side, int *fa_nodes) {
  GB_CHECK(path && sizes, "null argument");
  JkMesh M;
  const int r = read_jk(path, M);
  if (r < 0) return r;
  sizes[0] = M.nno;
  sizes[1] = M.nel;
  sizes[2] = (int)M.faces.size();
  if (xyz) memcpy(xyz, M.xyz.data(), M.xyz.size() * sizeof(double));
  if (el_nodes) memcpy(el_nodes, M.el.data(), M.el.size() * sizeof(int));
  for (size_t i = 0; i < M.faces.size(); i++) {
    const JkFace &f = M.faces[i];
    if (fa_type) fa_type[i] = f.type;
    if (fa_bc) fa_bc[i] = f.bc;
    if (fa_el) {
      fa_el[2 * i] = f.el1;
      fa_el[2 * i + 1] = f.el2;
    }
    if (fa_side) fa_side[i] = f.side1;
    if (fa_nodes)
      for (int k = 0; k < 4; k++) fa_nodes[4 * i + k] = f.nodes[k];
  }
  return 0;
}

int gbfem_write_field_std(const char *path, int nno, const int *dof_of_node, const double *x) {
  GB_CHECK(path && dof_of_node && x && nno > 0, "null argument");
  FILE *fp = fopen(path, "w");
  GB_CHECK(fp, std::string("cannot write ") + path);
  int n = 0;
  for (int v = 0; v < nno; v++) n += dof_of_node[v] >= 0;
  fprintf(fp, "%d %d\n", 1, 1);
  fprintf(fp, "%d\n", n);
  for (int v = 0; v < nno; v++) {
    if (dof_of_node[v] < 0) continue;
    fprintf(fp, "%d ", v + 1);
    fprintf(fp, "%.12lg ", x[dof_of_node[v]]);
    fprintf(fp, "\n");
  }
  const int bad = ferror(fp);
  fclose(fp);
  GB_CHECK(!bad, std::string("write error on ") + path);
  return n;
}

int gbfem_write_field_dg(const char *path, int nel, const int *p_el, const int *dof_off, const double *x,
                         int uniform) {
  GB_CHECK(path && p_el && dof_off && x && nel > 0, "null argument");
  FILE *fp = fopen(path, "w");
  GB_CHECK(fp, std::string("cannot write ") + path);
  fprintf(fp, "%d %d\n", 1, 1);
  for (int e = 0; e < (uniform ? 1 : nel); e++) fprintf(fp, "%d\n", -101 * p_el[e]);  // tensor basis: pdeg = 101 p
  for (int e = 0; e < nel; e++) {
    for (int i = dof_off[e]; i < dof_off[e + 1]; i++) fprintf(fp, "%.12lg ", std::fabs(x[i]) < 1e-15 ? 0.0 : x[i]);
    fprintf(fp, "\n");
  }
  const int bad = ferror(fp);
  fclose(fp);
  GB_CHECK(!bad, std::string("write error on ") + path);
  return nel;
}

}  // extern "C"

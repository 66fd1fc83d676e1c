// Host-side geometry builder: collects shapes, logical and placed volumes through the
// C-ABI, then `close()` flattens the hierarchy into device arrays (shape records, SoA
// transforms, daughter lists, per-volume BVH nodes in breadth-first complete-tree order,
// and the NavIndex table) and uploads them in one arena.
#pragma once
#include "vg_types.h"
#include <string>
#include <vector>

namespace vg {

struct HostShape {
  int32_t type = 0;
  std::vector<double> rec; // packed device record
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  int32_t left_pv = -1, right_pv = -1; // boolean operands
};

// Rigid transformation with the reference's flag semantics (Transformation3D.h:54-63).
struct HostXform {
  Xform m;
  bool has_trans = false, has_rot = false, identity = true;
  static HostXform Identity();
  static HostXform FromArrays(const double *t, const double *r);
  void MultiplyFromRight(HostXform const &rhs);
  void InverseTransform(const double *l, double *out) const;
};

struct HostPV {
  int32_t lv;
  HostXform xf;
  int32_t child = -1;
};

struct HostLV {
  int32_t shape;
  std::vector<int32_t> daughters;
};

struct HostBVH {
  int32_t depth = 0;
  std::vector<int32_t> prim, offset, nchild; // offset relative to the BVH's prim list
  std::vector<double> node_box;              // 6 per node
  std::vector<double> prim_box;              // 6 per daughter
};

class Geometry {
public:
  std::vector<HostShape> shapes;
  std::vector<HostLV> lvs;
  std::vector<HostPV> pvs;
  int32_t world = -1;
  bool closed   = false;
  int32_t max_depth = 0;

  // host copies of what was uploaded (kept for tests and the geometry blob)
  std::vector<HostBVH> bvhs;
  std::vector<int32_t> lv_bvh;
  std::vector<uint32_t> nav;
  size_t nav_words = 0;
  std::vector<float> shape_lbd_host; // FP32 shape descriptors (8 floats per shape) uploaded at close

  DevGeom dev{};
  void *arena      = nullptr;
  size_t arena_bytes = 0;
  int device       = -1;

  ~Geometry();
  int32_t add_shape(int32_t type, const double *p, int np, std::string &err);
  int32_t add_lv(int32_t shape, std::string &err);
  int32_t place(int32_t lv, const double *t, const double *r, int32_t mother_lv, std::string &err);
  int build_host(std::string &err); // daughter boxes, BVHs, NavIndex table (no GPU)
  int close(std::string &err);      // build_host if needed, then upload
  bool built = false;

  const double *shape_rec(int32_t s) const { return shapes[s].rec.data(); }

private:
  void build_bvh(int32_t lv, HostBVH &out) const;
  void daughter_box(int32_t pv, double *box6) const;
  void build_nav_table();
  int upload(std::string &err);
};

// Shape record builders (host; every transcendental the kernels need is evaluated here).
void make_box(const double *p, HostShape &s);
void make_tube(const double *p, HostShape &s);
void make_cone(const double *p, HostShape &s);
bool make_polycone(const double *p, int np, HostShape &s, std::string &err);
bool make_polyhedron(const double *p, int np, HostShape &s, std::string &err);
void make_torus2(const double *p, HostShape &s);
void make_trd(const double *p, HostShape &s);
bool make_trap(const double *p, int np, HostShape &s, std::string &err);

} // namespace vg

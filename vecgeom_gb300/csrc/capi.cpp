// extern "C" entry points declared in include/vecgeom_gb300.h.
#include "../../include/vecgeom_gb300.h"
#include "geom.h"
#include "launch.h"
#include "learn.h"
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <random>
#include <vector>
#include <new>
#include <string>

struct vg_geom {
  vg::Geometry geo;
  // device staging buffers of the host-pointer entry points (grown on demand, reused)
  std::mutex staging_mutex;
  void *staging       = nullptr;
  size_t staging_size = 0;
  vg::SortKeyParams sort{}; // set when the geometry is closed
  int queue_blocks = 1;     // work-queue kernel configuration: 1 = 256 x 1, 2 = 256 x 2, 3 = 128 x 3, 4 = 128 x 5;
                            // 5-8: the same budgets with the step split in two kernels (step, relocation)
                            // threads x resident blocks per SM
  // builder log for vg_geom_save / vg_geom_load: every successful builder call as
  // (op, arguments...) in call order, so a replay reproduces every id
  std::vector<double> oplog;
  const vg_mlp *proposer = nullptr; // learned proposal used by VG_NAV_LEARNED
  int propose_tensor      = 1;       // proposal kernel of VG_NAV_LEARNED: 1 tcgen05, 0 SIMT
  // host-pointer step: a copy stream and per-chunk events for overlapping the inputs'
  // host-to-device copies with the sort keys and proposals of the chunks already arrived
  static constexpr int kCopyChunks = 4;
  cudaStream_t copy_stream           = nullptr;
  cudaEvent_t chunk_ready[kCopyChunks] = {};
  cudaEvent_t steps_ready = nullptr, steps_copied = nullptr; // step lengths back while the relocation runs
  ~vg_geom()
  {
    if (staging) cudaFree(staging);
    for (cudaEvent_t ev : chunk_ready)
      if (ev) cudaEventDestroy(ev);
    if (steps_ready) cudaEventDestroy(steps_ready);
    if (steps_copied) cudaEventDestroy(steps_copied);
    if (copy_stream) cudaStreamDestroy(copy_stream);
  }
};

// Learned-proposal model: FP32 parameters + Adam state + BF16 inference copy, on the
// device of the geometry it was created for.
struct vg_mlp {
  int n_lv       = 0;
  size_t nparams = 0;
  float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr, *loss = nullptr;
  uint16_t *wbf = nullptr;
  float *ws = nullptr;
  size_t ws_floats = 0;
  uint32_t *idx = nullptr;
  size_t idx_n = 0;
  int t = 0;
  int *err = nullptr; // set by a tensor-core kernel whose bounded MMA wait gave up
  ~vg_mlp()
  {
    for (void *p : {(void *)params, (void *)grads, (void *)m, (void *)v, (void *)loss, (void *)wbf, (void *)ws,
                    (void *)idx, (void *)err})
      if (p) cudaFree(p);
  }
};

namespace {
thread_local std::string g_last_error;

int fail(int code, std::string const &msg)
{
  g_last_error = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char *what)
{
  return fail(VG_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
template <class T>
cudaError_t grow(T *&p, size_t &cap, size_t n)
{
  if (cap >= n && p) return cudaSuccess;
  if (p) cudaFree(p);
  p   = nullptr;
  cap = 0;
  const cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&p), (n ? n : 1) * sizeof(T));
  if (e == cudaSuccess) cap = n;
  return e;
}

bool built_ok(const vg_geom *g)
{
  if (!g) {
    g_last_error = "null geometry handle";
    return false;
  }
  if (!g->geo.built) {
    g_last_error = "geometry is not built (call vg_geom_build or vg_geom_close first)";
    return false;
  }
  return true;
}
bool closed_ok(const vg_geom *g)
{
  if (!g) {
    g_last_error = "null geometry handle";
    return false;
  }
  if (!g->geo.closed) {
    g_last_error = "geometry is not closed (call vg_geom_close first)";
    return false;
  }
  return true;
}
// Sort-key layout for VG_NAV_SORT: the logical-volume id in the high bits, then as many
// Morton bits per axis of the world box (the frame of global points) as fit in 32 bits.
vg::SortKeyParams sort_params(const vg::Geometry &geo, int cell_bits)
{
  vg::SortKeyParams p{};
  int lvb = 1;
  while (lvb < 31 && (size_t(1) << lvb) < geo.lvs.size()) ++lvb;
  p.lv_bits    = lvb;
  const int mx = (32 - lvb) / 3 > 10 ? 10 : (32 - lvb) / 3;
  p.cell_bits  = (cell_bits > 0 && cell_bits < mx) ? cell_bits : mx;
  const vg::HostShape &ws = geo.shapes[geo.lvs[geo.pvs[geo.world].lv].shape];
  for (int k = 0; k < 3; ++k) {
    const double ext = ws.hi[k] - ws.lo[k];
    p.lo[k]          = (float)ws.lo[k];
    p.scale[k]       = ext > 0. ? (float)((double)(1u << p.cell_bits) / ext) : 0.f;
  }
  return p;
}

constexpr uint32_t kNavFlags = VG_PREC_MIXED | VG_NAV_SORT | VG_NAV_QUEUE | VG_NAV_LEARNED;

size_t step_workspace_bytes(size_t n, uint32_t flags)
{
  size_t b = 0;
  if (flags & VG_NAV_QUEUE) b += 256 + ((3 * n * sizeof(double) + 255) & ~size_t(255));
  if (flags & VG_NAV_LEARNED) b += (n + 255) & ~size_t(255);
  if (flags & VG_NAV_SORT) b += vg::nav_sort_workspace_bytes(n);
  return b;
}

// Workspace of a scheduled step: work-queue counter (256 bytes) and the relocation points
// of the split step (3 n doubles, in visiting order) with VG_NAV_QUEUE, proposal slots (n
// bytes) with VG_NAV_LEARNED, then the sort arrays (keys first).
struct StepWs {
  unsigned long long *counter = nullptr;
  double *reloc               = nullptr;
  int8_t *slots               = nullptr;
  unsigned char *sort         = nullptr;
};
StepWs step_ws(void *ws, size_t n, uint32_t flags)
{
  StepWs r;
  unsigned char *w = static_cast<unsigned char *>(ws);
  if (flags & VG_NAV_QUEUE) {
    r.counter = reinterpret_cast<unsigned long long *>(w);
    w += 256;
    r.reloc = reinterpret_cast<double *>(w);
    w += (3 * n * sizeof(double) + 255) & ~size_t(255);
  }
  if (flags & VG_NAV_LEARNED) {
    r.slots = reinterpret_cast<int8_t *>(w);
    w += (n + 255) & ~size_t(255);
  }
  r.sort = w;
  return r;
}

cudaError_t propose_launch(const vg_geom *g, const vg::StepArgs &a, int8_t *slots, cudaStream_t s)
{
  // proposals are stored per track, so they are computed in track order: coalesced input
  // loads beat the geometry locality of the sorted order
  vg::StepArgs pa = a;
  pa.order        = nullptr;
  return g->propose_tensor ? vg::launch_mlp_propose_tc(g->geo.dev, pa, g->proposer->wbf, slots, g->proposer->err, s)
                           : vg::launch_mlp_propose(g->geo.dev, pa, g->proposer->wbf, slots, s);
}

// Validated step launch with optional sort and work queue; `ws` holds the counter
// (256 bytes, first) and the sort arrays. prepared: the sort keys and proposals of all
// tracks are already in the workspace (the pipelined host-pointer entry point).
int step_launch(const vg_geom *g, vg::StepArgs a, uint32_t flags, void *ws, size_t ws_bytes, cudaStream_t s,
                bool prepared = false)
{
  if (flags & ~kNavFlags) return fail(VG_EINVAL, "invalid navigation flags");
  if ((flags & (VG_NAV_QUEUE | VG_NAV_LEARNED)) && !(flags & VG_PREC_MIXED))
    return fail(VG_EINVAL, "VG_NAV_QUEUE and VG_NAV_LEARNED need VG_PREC_MIXED");
  if ((flags & VG_NAV_LEARNED) && !g->proposer) return fail(VG_ESTATE, "VG_NAV_LEARNED without a proposer model");
  if (a.n > 0xffffffffull) return fail(VG_EINVAL, "more than 2^32-1 tracks in one call");
  const size_t need = step_workspace_bytes(a.n, flags);
  if (need > 0 && (!ws || ws_bytes < need || (reinterpret_cast<uintptr_t>(ws) & 255u)))
    return fail(VG_EINVAL, "workspace missing, too small or not 256-byte aligned");
  const StepWs w = step_ws(ws, a.n, flags);
  unsigned long long *counter = w.counter;
  cudaError_t e = cudaSuccess;
  if (flags & VG_NAV_SORT) {
    const uint32_t *order = nullptr;
    e = vg::launch_nav_sort(g->geo.dev, g->sort, a.x, a.y, a.z, a.in, a.n, w.sort, &order, s, nullptr, prepared);
    if (e != cudaSuccess) return cuda_fail(e, "track sort launch");
    a.order = order;
  }
  if (flags & VG_NAV_LEARNED) {
    if (!prepared) {
      e = propose_launch(g, a, w.slots, s);
      if (e != cudaSuccess) return cuda_fail(e, "proposal launch");
    }
    a.proposal = w.slots;
  }
  if (flags & VG_NAV_QUEUE) {
    a.reloc = w.reloc;
    e       = vg::launch_step_mixed_queue(g->geo.dev, a, counter, g->queue_blocks, s);
  }
  else
    e = vg::launch_step(g->geo.dev, a, flags & VG_PREC_MIXED, s);
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "navigation step launch");
}

enum GeomOp { kOpShape = 1, kOpLv = 2, kOpPlace = 3, kOpWorld = 4 };

int32_t add_shape(vg_geom *g, int type, const double *p, int np)
{
  if (!g) return fail(VG_EINVAL, "null geometry handle");
  std::string err;
  const int32_t id = g->geo.add_shape(type, p, np, err);
  if (id < 0) return fail(g->geo.closed ? VG_ESTATE : VG_EINVAL, err);
  g->oplog.insert(g->oplog.end(), {(double)kOpShape, (double)type, (double)np});
  g->oplog.insert(g->oplog.end(), p, p + np);
  return id;
}

enum Query { kQInside = 0, kQContains = 1, kQDistIn = 2, kQDistOut = 3, kQSafIn = 4, kQSafOut = 5 };

// One SoA query of shape `shape`; the points go through `xf` first when apply_xf is set
// (placed volumes), or are in the shape's own frame (unplaced queries).
int shape_query(const vg_geom *g, int32_t shape, const vg::Xform &xf, int apply_xf, int q, const double *x,
                const double *y, const double *z, const double *dx, const double *dy, const double *dz, size_t n,
                void *out, uint32_t flags, void *stream)
{
  vg::Geometry const &geo = g->geo;
  if (flags > VG_PREC_MIXED) return fail(VG_EINVAL, "invalid precision flags");
  if (n > 0 && (!x || !y || !z || !out || ((q == kQDistIn || q == kQDistOut) && (!dx || !dy || !dz))))
    return fail(VG_EINVAL, "null input/output array");
  const int32_t type = geo.shapes[shape].type;
  vg::QueryArgs a{x, y, z, dx, dy, dz, n, out};
  const bool composite = type == vg::kShapePolycone || type == vg::kShapePolyhedron || type == vg::kShapeBoolMinus;
  const bool mixed      = (flags & VG_PREC_MIXED) != 0;
  const float *lbd      = mixed ? geo.shape_lbd_host.data() + 8 * (size_t)shape : nullptr;
  const cudaError_t e   = composite ? vg::launch_shape_query_dyn_fp64(geo.dev, shape, type, xf, apply_xf, q, a,
                                                                    (cudaStream_t)stream, mixed)
                                  : vg::launch_shape_query_fp64(type, geo.shape_rec(shape), xf, apply_xf, q, a,
                                                                (cudaStream_t)stream, lbd);
  if (e == cudaErrorNotSupported) return fail(VG_EINVAL, "shape type not supported by this query path");
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "shape query launch");
}

int placed_query(const vg_geom *g, int32_t pv, int q, const double *x, const double *y, const double *z,
                 const double *dx, const double *dy, const double *dz, size_t n, void *out, uint32_t flags,
                 void *stream)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  vg::Geometry const &geo = g->geo;
  if (pv < 0 || pv >= (int32_t)geo.pvs.size()) return fail(VG_EINVAL, "invalid placed-volume id");
  return shape_query(g, geo.lvs[geo.pvs[pv].lv].shape, geo.pvs[pv].xf.m, 1, q, x, y, z, dx, dy, dz, n, out, flags,
                     stream);
}

int unplaced_query(const vg_geom *g, int32_t shape, int q, const double *x, const double *y, const double *z,
                   const double *dx, const double *dy, const double *dz, size_t n, void *out, uint32_t flags,
                   void *stream)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  if (shape < 0 || shape >= (int32_t)g->geo.shapes.size()) return fail(VG_EINVAL, "invalid shape id");
  return shape_query(g, shape, vg::Xform{}, 0, q, x, y, z, dx, dy, dz, n, out, flags, stream);
}
} // namespace

extern "C" {

const char *vg_last_error(void) { return g_last_error.c_str(); }
const char *vg_version(void) { return "vecgeom_gb300 0.1 (sm_103a)"; }

int vg_geom_create(vg_geom **out)
{
  if (!out) return fail(VG_EINVAL, "null output pointer");
  *out = new (std::nothrow) vg_geom();
  return *out ? VG_OK : fail(VG_ENOMEM, "out of host memory");
}
void vg_geom_destroy(vg_geom *g) { delete g; }

int32_t vg_geom_add_box(vg_geom *g, double dx, double dy, double dz)
{
  const double p[3] = {dx, dy, dz};
  return add_shape(g, vg::kShapeBox, p, 3);
}
int32_t vg_geom_add_tube(vg_geom *g, double rmin, double rmax, double dz, double sphi, double dphi)
{
  const double p[5] = {rmin, rmax, dz, sphi, dphi};
  return add_shape(g, vg::kShapeTube, p, 5);
}
int32_t vg_geom_add_cone(vg_geom *g, double rmin1, double rmax1, double rmin2, double rmax2, double dz, double sphi,
                         double dphi)
{
  const double p[7] = {rmin1, rmax1, rmin2, rmax2, dz, sphi, dphi};
  return add_shape(g, vg::kShapeCone, p, 7);
}
int32_t vg_geom_add_polycone(vg_geom *g, double sphi, double dphi, int32_t nz, const double *z, const double *rmin,
                             const double *rmax)
{
  if (nz < 2 || nz > 1024 || !z || !rmin || !rmax) return fail(VG_EINVAL, "polycone needs 2..1024 z planes");
  std::vector<double> p{sphi, dphi, (double)nz};
  p.insert(p.end(), z, z + nz);
  p.insert(p.end(), rmin, rmin + nz);
  p.insert(p.end(), rmax, rmax + nz);
  return add_shape(g, vg::kShapePolycone, p.data(), (int)p.size());
}
int32_t vg_geom_add_polyhedron(vg_geom *g, double phistart, double phidelta, int32_t nsides, int32_t nz,
                               const double *z, const double *rmin, const double *rmax)
{
  if (nz < 2 || nz > 1024 || nsides < 1 || nsides > 1024 || !z || !rmin || !rmax)
    return fail(VG_EINVAL, "polyhedron needs 2..1024 z planes and 1..1024 sides");
  std::vector<double> p{phistart, phidelta, (double)nsides, (double)nz};
  p.insert(p.end(), z, z + nz);
  p.insert(p.end(), rmin, rmin + nz);
  p.insert(p.end(), rmax, rmax + nz);
  return add_shape(g, vg::kShapePolyhedron, p.data(), (int)p.size());
}
int32_t vg_geom_add_torus2(vg_geom *g, double rmin, double rmax, double rtor, double sphi, double dphi)
{
  const double p[5] = {rmin, rmax, rtor, sphi, dphi};
  return add_shape(g, vg::kShapeTorus2, p, 5);
}
int32_t vg_geom_add_trd(vg_geom *g, double dx1, double dx2, double dy1, double dy2, double dz)
{
  const double p[5] = {dx1, dx2, dy1, dy2, dz};
  return add_shape(g, vg::kShapeTrd, p, 5);
}
int32_t vg_geom_add_trap(vg_geom *g, double dz, double theta, double phi, double dy1, double dx1, double dx2,
                         double alpha1, double dy2, double dx3, double dx4, double alpha2)
{
  const double p[11] = {dz, theta, phi, dy1, dx1, dx2, alpha1, dy2, dx3, dx4, alpha2};
  return add_shape(g, vg::kShapeTrap, p, 11);
}
int32_t vg_geom_add_sphere(vg_geom *g, double rmin, double rmax, double sphi, double dphi, double stheta,
                           double dtheta)
{
  const double p[6] = {rmin, rmax, sphi, dphi, stheta, dtheta};
  return add_shape(g, vg::kShapeSphere, p, 6);
}
int32_t vg_geom_add_hype(vg_geom *g, double rmin, double rmax, double stereo_in, double stereo_out, double dz)
{
  const double p[5] = {rmin, rmax, stereo_in, stereo_out, dz};
  return add_shape(g, vg::kShapeHype, p, 5);
}
int32_t vg_geom_add_gentrap(vg_geom *g, const double *vertices_x, const double *vertices_y, double dz)
{
  if (!vertices_x || !vertices_y) return fail(VG_EINVAL, "null vertex array");
  double p[17];
  for (int i = 0; i < 8; ++i) p[i] = vertices_x[i], p[8 + i] = vertices_y[i];
  p[16] = dz;
  return add_shape(g, vg::kShapeGenTrap, p, 17);
}
int32_t vg_geom_add_cut_tube(vg_geom *g, double rmin, double rmax, double dz, double sphi, double dphi, double bx,
                             double by, double bz, double tx, double ty, double tz)
{
  const double p[11] = {rmin, rmax, dz, sphi, dphi, bx, by, bz, tx, ty, tz};
  return add_shape(g, vg::kShapeCutTube, p, 11);
}
int32_t vg_geom_add_trap_corners(vg_geom *g, const double *corners)
{
  if (!corners) return fail(VG_EINVAL, "null corner array");
  return add_shape(g, vg::kShapeTrap, corners, 24);
}
int32_t vg_geom_add_trap_planes(vg_geom *g, double dz, const double *planes)
{
  if (!planes) return fail(VG_EINVAL, "null plane array");
  double p[17];
  p[0] = dz;
  for (int i = 0; i < 16; ++i) p[1 + i] = planes[i];
  return add_shape(g, vg::kShapeTrap, p, 17);
}
int32_t vg_geom_add_boolean_subtraction(vg_geom *g, int32_t left_pv, int32_t right_pv)
{
  const double p[2] = {(double)left_pv, (double)right_pv};
  return add_shape(g, vg::kShapeBoolMinus, p, 2);
}

int32_t vg_geom_add_logical_volume(vg_geom *g, int32_t shape_id)
{
  if (!g) return fail(VG_EINVAL, "null geometry handle");
  std::string err;
  const int32_t id = g->geo.add_lv(shape_id, err);
  if (id < 0) return fail(g->geo.closed ? VG_ESTATE : VG_EINVAL, err);
  g->oplog.insert(g->oplog.end(), {(double)kOpLv, (double)shape_id});
  return id;
}
static void log_place(vg_geom *g, int32_t lv, int32_t mother, const double *trans, const double *rot)
{
  g->oplog.insert(g->oplog.end(), {(double)kOpPlace, (double)lv, (double)mother});
  g->oplog.insert(g->oplog.end(), trans, trans + 3);
  g->oplog.insert(g->oplog.end(), rot, rot + 9);
}
int32_t vg_geom_place(vg_geom *g, int32_t lv, const double trans[3], const double rot[9])
{
  if (!g || !trans || !rot) return fail(VG_EINVAL, "null argument");
  std::string err;
  const int32_t id = g->geo.place(lv, trans, rot, -1, err);
  if (id < 0) return fail(g->geo.closed ? VG_ESTATE : VG_EINVAL, err);
  log_place(g, lv, -1, trans, rot);
  return id;
}
int32_t vg_geom_place_daughter(vg_geom *g, int32_t mother_lv, int32_t lv, const double trans[3], const double rot[9])
{
  if (!g || !trans || !rot) return fail(VG_EINVAL, "null argument");
  if (mother_lv < 0) return fail(VG_EINVAL, "invalid mother logical volume id");
  std::string err;
  const int32_t id = g->geo.place(lv, trans, rot, mother_lv, err);
  if (id < 0) return fail(g->geo.closed ? VG_ESTATE : VG_EINVAL, err);
  log_place(g, lv, mother_lv, trans, rot);
  return id;
}
int vg_geom_set_world(vg_geom *g, int32_t world_pv)
{
  if (!g) return fail(VG_EINVAL, "null geometry handle");
  if (g->geo.closed) return fail(VG_ESTATE, "geometry is closed");
  if (world_pv < 0 || world_pv >= (int32_t)g->geo.pvs.size()) return fail(VG_EINVAL, "invalid placed-volume id");
  g->geo.world = world_pv;
  g->oplog.insert(g->oplog.end(), {(double)kOpWorld, (double)world_pv});
  return VG_OK;
}

static const char kGeomMagic[8] = {'V', 'G', 'G', 'B', '3', '0', '0', 'G'};
constexpr uint32_t kGeomVersion  = 1;

int vg_geom_save(const vg_geom *g, const char *path)
{
  if (!g || !path) return fail(VG_EINVAL, "null argument");
  FILE *f = std::fopen(path, "wb");
  if (!f) return fail(VG_EINVAL, std::string("cannot open ") + path + " for writing");
  const uint64_t n = g->oplog.size();
  bool ok = std::fwrite(kGeomMagic, 1, 8, f) == 8 && std::fwrite(&kGeomVersion, 4, 1, f) == 1 &&
            std::fwrite(&n, 8, 1, f) == 1 && (n == 0 || std::fwrite(g->oplog.data(), 8, n, f) == n);
  ok = (std::fclose(f) == 0) && ok;
  return ok ? VG_OK : fail(VG_EINVAL, std::string("write error on ") + path);
}

int vg_geom_load(vg_geom *g, const char *path)
{
  if (!g || !path) return fail(VG_EINVAL, "null argument");
  if (!g->oplog.empty() || !g->geo.shapes.empty() || g->geo.closed)
    return fail(VG_ESTATE, "vg_geom_load needs a new, empty geometry");
  FILE *f = std::fopen(path, "rb");
  if (!f) return fail(VG_EINVAL, std::string("cannot open ") + path);
  char magic[8];
  uint32_t version = 0;
  uint64_t n       = 0;
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kGeomMagic, 8) == 0 &&
            std::fread(&version, 4, 1, f) == 1 && version == kGeomVersion && std::fread(&n, 8, 1, f) == 1 &&
            n < (uint64_t(1) << 34);
  std::vector<double> log;
  if (ok) {
    log.resize(n);
    ok = n == 0 || std::fread(log.data(), 8, n, f) == n;
  }
  std::fclose(f);
  if (!ok) return fail(VG_EINVAL, std::string("not a saved geometry (or truncated): ") + path);
  size_t i = 0;
  auto take = [&](size_t k) { return i + k <= log.size(); };
  while (i < log.size()) {
    const int op = (int)log[i];
    int32_t r    = -1;
    if (op == kOpShape && take(3) && take(3 + (size_t)log[i + 2])) {
      const int np = (int)log[i + 2];
      r            = add_shape(g, (int)log[i + 1], log.data() + i + 3, np);
      i += 3 + np;
    } else if (op == kOpLv && take(2)) {
      r = vg_geom_add_logical_volume(g, (int32_t)log[i + 1]);
      i += 2;
    } else if (op == kOpPlace && take(15)) {
      const int32_t lv = (int32_t)log[i + 1], mother = (int32_t)log[i + 2];
      r = mother < 0 ? vg_geom_place(g, lv, log.data() + i + 3, log.data() + i + 6)
                     : vg_geom_place_daughter(g, mother, lv, log.data() + i + 3, log.data() + i + 6);
      i += 15;
    } else if (op == kOpWorld && take(2)) {
      r = vg_geom_set_world(g, (int32_t)log[i + 1]);
      i += 2;
    } else {
      return fail(VG_EINVAL, std::string("corrupt saved geometry: ") + path);
    }
    if (r < 0) return r;
  }
  return VG_OK;
}
int vg_geom_close(vg_geom *g)
{
  if (!g) return fail(VG_EINVAL, "null geometry handle");
  std::string err;
  if (g->geo.close(err) != 0) return fail(g->geo.closed ? VG_ESTATE : VG_ECUDA, err);
  if (g->geo.world >= 0) g->sort = sort_params(g->geo, 0);
  return VG_OK;
}
int vg_geom_build(vg_geom *g)
{
  if (!g) return fail(VG_EINVAL, "null geometry handle");
  std::string err;
  if (g->geo.build_host(err) != 0) return fail(g->geo.closed ? VG_ESTATE : VG_EINVAL, err);
  return VG_OK;
}
int vg_geom_info(const vg_geom *g, int32_t *n_shapes, int32_t *n_lv, int32_t *n_pv, int32_t *max_depth,
                 size_t *nav_table_words, size_t *device_bytes)
{
  if (!g) return fail(VG_EINVAL, "null geometry handle");
  if (n_shapes) *n_shapes = (int32_t)g->geo.shapes.size();
  if (n_lv) *n_lv = (int32_t)g->geo.lvs.size();
  if (n_pv) *n_pv = (int32_t)g->geo.pvs.size();
  if (max_depth) *max_depth = g->geo.max_depth;
  if (nav_table_words) *nav_table_words = g->geo.nav_words;
  if (device_bytes) *device_bytes = g->geo.arena_bytes;
  return VG_OK;
}
int vg_geom_nav_table(const vg_geom *g, uint32_t *out, size_t words)
{
  if (!built_ok(g)) return VG_ESTATE;
  if (!out || words < g->geo.nav_words) return fail(VG_EINVAL, "output buffer too small");
  std::memcpy(out, g->geo.nav.data(), g->geo.nav_words * sizeof(uint32_t));
  return VG_OK;
}
int vg_geom_bvh_sizes(const vg_geom *g, int32_t lv, int32_t *n_nodes, int32_t *n_prims, int32_t *depth)
{
  if (!built_ok(g)) return VG_ESTATE;
  if (lv < 0 || lv >= (int32_t)g->geo.lvs.size() || g->geo.lv_bvh[lv] < 0)
    return fail(VG_EINVAL, "logical volume has no BVH");
  vg::HostBVH const &b = g->geo.bvhs[g->geo.lv_bvh[lv]];
  *n_nodes = (int32_t)b.nchild.size();
  *n_prims = (int32_t)b.prim.size();
  *depth   = b.depth;
  return VG_OK;
}
int vg_geom_bvh_arrays(const vg_geom *g, int32_t lv, int32_t *prim_id, int32_t *offset, int32_t *nchild,
                       double *node_box6, double *prim_box6)
{
  if (!built_ok(g)) return VG_ESTATE;
  if (lv < 0 || lv >= (int32_t)g->geo.lvs.size() || g->geo.lv_bvh[lv] < 0)
    return fail(VG_EINVAL, "logical volume has no BVH");
  vg::HostBVH const &b = g->geo.bvhs[g->geo.lv_bvh[lv]];
  std::memcpy(prim_id, b.prim.data(), b.prim.size() * sizeof(int32_t));
  std::memcpy(offset, b.offset.data(), b.offset.size() * sizeof(int32_t));
  std::memcpy(nchild, b.nchild.data(), b.nchild.size() * sizeof(int32_t));
  std::memcpy(node_box6, b.node_box.data(), b.node_box.size() * sizeof(double));
  std::memcpy(prim_box6, b.prim_box.data(), b.prim_box.size() * sizeof(double));
  return VG_OK;
}
int vg_geom_shape_extent(const vg_geom *g, int32_t shape_id, double lo[3], double hi[3])
{
  if (!g || shape_id < 0 || shape_id >= (int32_t)g->geo.shapes.size()) return fail(VG_EINVAL, "invalid shape id");
  for (int k = 0; k < 3; ++k) lo[k] = g->geo.shapes[shape_id].lo[k], hi[k] = g->geo.shapes[shape_id].hi[k];
  return VG_OK;
}

int vg_placed_inside(const vg_geom *g, int32_t pv, const double *x, const double *y, const double *z, size_t n,
                     int32_t *out, uint32_t flags, void *stream)
{
  return placed_query(g, pv, kQInside, x, y, z, nullptr, nullptr, nullptr, n, out, flags, stream);
}
int vg_placed_contains(const vg_geom *g, int32_t pv, const double *x, const double *y, const double *z, size_t n,
                       uint8_t *out, uint32_t flags, void *stream)
{
  return placed_query(g, pv, kQContains, x, y, z, nullptr, nullptr, nullptr, n, out, flags, stream);
}
int vg_placed_distance_to_in(const vg_geom *g, int32_t pv, const double *x, const double *y, const double *z,
                             const double *dx, const double *dy, const double *dz, const double *step_max, size_t n,
                             double *out, uint32_t flags, void *stream)
{
  (void)step_max;
  return placed_query(g, pv, kQDistIn, x, y, z, dx, dy, dz, n, out, flags, stream);
}
int vg_placed_distance_to_out(const vg_geom *g, int32_t pv, const double *x, const double *y, const double *z,
                              const double *dx, const double *dy, const double *dz, const double *step_max, size_t n,
                              double *out, uint32_t flags, void *stream)
{
  (void)step_max;
  return placed_query(g, pv, kQDistOut, x, y, z, dx, dy, dz, n, out, flags, stream);
}
int vg_placed_safety_to_in(const vg_geom *g, int32_t pv, const double *x, const double *y, const double *z, size_t n,
                           double *out, uint32_t flags, void *stream)
{
  return placed_query(g, pv, kQSafIn, x, y, z, nullptr, nullptr, nullptr, n, out, flags, stream);
}
int vg_placed_safety_to_out(const vg_geom *g, int32_t pv, const double *x, const double *y, const double *z, size_t n,
                            double *out, uint32_t flags, void *stream)
{
  return placed_query(g, pv, kQSafOut, x, y, z, nullptr, nullptr, nullptr, n, out, flags, stream);
}

int vg_shape_inside(const vg_geom *g, int32_t shape, const double *x, const double *y, const double *z, size_t n,
                    int32_t *out, uint32_t flags, void *stream)
{
  return unplaced_query(g, shape, kQInside, x, y, z, nullptr, nullptr, nullptr, n, out, flags, stream);
}
int vg_shape_contains(const vg_geom *g, int32_t shape, const double *x, const double *y, const double *z, size_t n,
                      uint8_t *out, uint32_t flags, void *stream)
{
  return unplaced_query(g, shape, kQContains, x, y, z, nullptr, nullptr, nullptr, n, out, flags, stream);
}
int vg_shape_distance_to_in(const vg_geom *g, int32_t shape, const double *x, const double *y, const double *z,
                            const double *dx, const double *dy, const double *dz, const double *step_max, size_t n,
                            double *out, uint32_t flags, void *stream)
{
  (void)step_max;
  return unplaced_query(g, shape, kQDistIn, x, y, z, dx, dy, dz, n, out, flags, stream);
}
int vg_shape_distance_to_out(const vg_geom *g, int32_t shape, const double *x, const double *y, const double *z,
                             const double *dx, const double *dy, const double *dz, const double *step_max, size_t n,
                             double *out, uint32_t flags, void *stream)
{
  (void)step_max;
  return unplaced_query(g, shape, kQDistOut, x, y, z, dx, dy, dz, n, out, flags, stream);
}
int vg_shape_safety_to_in(const vg_geom *g, int32_t shape, const double *x, const double *y, const double *z,
                          size_t n, double *out, uint32_t flags, void *stream)
{
  return unplaced_query(g, shape, kQSafIn, x, y, z, nullptr, nullptr, nullptr, n, out, flags, stream);
}
int vg_shape_safety_to_out(const vg_geom *g, int32_t shape, const double *x, const double *y, const double *z,
                           size_t n, double *out, uint32_t flags, void *stream)
{
  return unplaced_query(g, shape, kQSafOut, x, y, z, nullptr, nullptr, nullptr, n, out, flags, stream);
}

int vg_nav_locate_point(const vg_geom *g, const double *x, const double *y, const double *z, size_t n,
                        vg_navstate *out, void *stream)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  if (g->geo.world < 0) return fail(VG_ESTATE, "geometry has no world volume");
  if (n > 0 && (!x || !y || !z || !out)) return fail(VG_EINVAL, "null input/output array");
  const cudaError_t e = vg::launch_locate_fp64(g->geo.dev, x, y, z, n, reinterpret_cast<vg::NavState *>(out),
                                               (cudaStream_t)stream);
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "locate launch");
}

int vg_nav_approach_next_daughter(const vg_geom *g, const double *x, const double *y, const double *z,
                                  const double *dx, const double *dy, const double *dz, const vg_navstate *in,
                                  double *step, int32_t *status, size_t n, void *stream)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  if (n > 0 && (!x || !y || !z || !dx || !dy || !dz || !in || !step))
    return fail(VG_EINVAL, "null input/output array");
  const cudaError_t e =
      vg::launch_approach_fp64(g->geo.dev, x, y, z, dx, dy, dz, reinterpret_cast<const vg::NavState *>(in), step,
                               status, n, (cudaStream_t)stream);
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "approach launch");
}

int vg_nav_compute_step_and_next_volume(const vg_geom *g, const double *x, const double *y, const double *z,
                                        const double *dx, const double *dy, const double *dz,
                                        const double *step_limit, const vg_navstate *in, vg_navstate *out,
                                        double *step, int32_t *status, size_t n, uint32_t flags, void *stream)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  if (g->geo.world < 0) return fail(VG_ESTATE, "geometry has no world volume");
  if (flags > VG_PREC_MIXED)
    return fail(VG_EINVAL, "invalid precision flags (scheduling flags need vg_nav_compute_step_and_next_volume_ws)");
  return vg_nav_compute_step_and_next_volume_ws(g, x, y, z, dx, dy, dz, step_limit, in, out, step, status, nullptr, n,
                                                flags, nullptr, 0, stream);
}

size_t vg_nav_step_workspace_bytes(size_t n, uint32_t flags) { return step_workspace_bytes(n, flags); }

int vg_nav_compute_step_and_next_volume_ws(const vg_geom *g, const double *x, const double *y, const double *z,
                                           const double *dx, const double *dy, const double *dz,
                                           const double *step_limit, const vg_navstate *in, vg_navstate *out,
                                           double *step, int32_t *status, int32_t *nodes_visited, size_t n,
                                           uint32_t flags, void *workspace, size_t workspace_bytes, void *stream)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  if (g->geo.world < 0) return fail(VG_ESTATE, "geometry has no world volume");
  if (n > 0 && (!x || !y || !z || !dx || !dy || !dz || !in || !out || !step))
    return fail(VG_EINVAL, "null input/output array");
  vg::StepArgs a{x,   y,   z,   dx,  dy,  dz, step_limit, reinterpret_cast<const vg::NavState *>(in),
                 reinterpret_cast<vg::NavState *>(out), step, status, nodes_visited, n};
  return step_launch(g, a, flags, workspace, workspace_bytes, (cudaStream_t)stream);
}

size_t transport_ws_bytes(size_t n, uint32_t flags)
{
  const size_t a = (n * sizeof(uint32_t) + 255) & ~size_t(255);
  size_t b       = 2 * a + 4 * 256; // two track lists, two counts, queue counter, loop control
  if (flags & VG_NAV_LEARNED) b += (n + 255) & ~size_t(255);
  if (flags & VG_NAV_SORT) b += vg::nav_sort_workspace_bytes(n);
  return b;
}

size_t vg_nav_transport_workspace_bytes(size_t n, uint32_t flags) { return transport_ws_bytes(n, flags); }

int vg_nav_transport(const vg_geom *g, double *x, double *y, double *z, const double *dx, const double *dy,
                     const double *dz, vg_navstate *states, size_t n, int32_t max_steps, uint32_t flags,
                     int32_t *nsteps, int32_t *status, vg_navstate *trace_states, double *trace_steps,
                     size_t trace_tracks, int32_t *iterations, void *workspace, size_t workspace_bytes, void *stream)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  if (g->geo.world < 0) return fail(VG_ESTATE, "geometry has no world volume");
  if (flags & ~kNavFlags) return fail(VG_EINVAL, "invalid navigation flags");
  if ((flags & (VG_NAV_QUEUE | VG_NAV_LEARNED)) && !(flags & VG_PREC_MIXED))
    return fail(VG_EINVAL, "VG_NAV_QUEUE and VG_NAV_LEARNED need VG_PREC_MIXED");
  if ((flags & VG_NAV_LEARNED) && !g->proposer) return fail(VG_ESTATE, "VG_NAV_LEARNED without a proposer model");
  if (n > 0xffffffffull || max_steps < 0) return fail(VG_EINVAL, "n or max_steps out of range");
  if (n > 0 && (!x || !y || !z || !dx || !dy || !dz || !states || !nsteps || !status))
    return fail(VG_EINVAL, "null input/output array");
  if (trace_tracks > 0 && (!trace_states || !trace_steps)) return fail(VG_EINVAL, "null trace arrays");
  if (trace_tracks > n) trace_tracks = n;
  const size_t need = transport_ws_bytes(n, flags);
  if (!workspace || workspace_bytes < need || (reinterpret_cast<uintptr_t>(workspace) & 255u))
    return fail(VG_EINVAL, "workspace missing, too small or not 256-byte aligned");
  if (iterations) *iterations = 0;
  if (n == 0) return VG_OK;
  cudaStream_t s   = (cudaStream_t)stream;
  unsigned char *w = static_cast<unsigned char *>(workspace);
  const size_t al  = (n * sizeof(uint32_t) + 255) & ~size_t(255);
  uint32_t *list[2] = {reinterpret_cast<uint32_t *>(w), reinterpret_cast<uint32_t *>(w + al)};
  unsigned int *cnt[2] = {reinterpret_cast<unsigned int *>(w + 2 * al), reinterpret_cast<unsigned int *>(w + 2 * al + 256)};
  unsigned long long *counter = reinterpret_cast<unsigned long long *>(w + 2 * al + 512);
  unsigned char *rest         = w + 2 * al + 1024;
  int8_t *slots               = nullptr;
  if (flags & VG_NAV_LEARNED) {
    slots = reinterpret_cast<int8_t *>(rest);
    rest += (n + 255) & ~size_t(255);
  }
  vg::NavState *st = reinterpret_cast<vg::NavState *>(states);
  cudaError_t e    = vg::launch_transport_init(st, n, nsteps, status, list[0], cnt[0], s);
  // With VG_NAV_QUEUE, once fewer tracks are alive than the GPU holds threads of the tail
  // kernel, the rest of the stream runs as one refill pass (launch_transport_drain).
  unsigned int drain_below = 0;
  if (flags & VG_NAV_QUEUE) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess)
      drain_below = (unsigned int)sms * 512u;
  }
  // The iterations run in a device-side loop (a CUDA graph with a while-node, no host round
  // trip per iteration); the host reads the loop's end state once and runs the tail pass.
  vg::TransportCtl *ctl = reinterpret_cast<vg::TransportCtl *>(w + 2 * al + 768);
  vg::TransportLoop L{};
  L.g     = &g->geo.dev;
  L.ta    = vg::TransportArgs{x,       y,           z,       dx,          dy,         dz,    st,
                           nsteps,  status,      (int)max_steps, reinterpret_cast<vg::NavState *>(trace_states),
                           trace_steps, trace_tracks, nullptr, 0, nullptr, nullptr, nullptr};
  L.n     = n;
  L.list[0] = list[0], L.list[1] = list[1];
  L.cnt[0] = cnt[0], L.cnt[1] = cnt[1];
  L.counter        = counter;
  L.ctl            = ctl;
  L.mixed          = (flags & VG_PREC_MIXED) != 0;
  L.queue_blocks   = g->queue_blocks;
  L.sort_on        = (flags & VG_NAV_SORT) != 0;
  L.sort           = g->sort;
  L.sort_ws        = rest;
  L.slots          = slots;
  L.propose_tensor = g->propose_tensor;
  L.wbf            = (flags & VG_NAV_LEARNED) ? g->proposer->wbf : nullptr;
  L.mlp_err        = (flags & VG_NAV_LEARNED) ? g->proposer->err : nullptr;
  L.max_steps      = (int)max_steps;
  L.drain_below    = drain_below;
  vg::TransportCtl end{};
  if (e == cudaSuccess) e = vg::run_transport_loop(L, s, &end);
  int it = end.it;
  if (e == cudaSuccess && end.live > 0 && end.live < drain_below && it < max_steps) {
    vg::TransportArgs ta{x,       y,           z,       dx,          dy,         dz,    st,
                         nsteps,  status,      (int)max_steps, reinterpret_cast<vg::NavState *>(trace_states),
                         trace_steps, trace_tracks, list[end.cur], end.live, nullptr, nullptr, nullptr};
    e = vg::launch_transport_drain(g->geo.dev, ta, (flags & VG_PREC_MIXED) != 0, counter, s);
    ++it;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (iterations) *iterations = it;
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "transport stream");
}

int vg_nav_sort_tracks(const vg_geom *g, const double *x, const double *y, const double *z, const vg_navstate *in,
                       size_t n, uint32_t *order, uint32_t *keys, void *workspace, size_t workspace_bytes,
                       void *stream)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  if (g->geo.world < 0) return fail(VG_ESTATE, "geometry has no world volume");
  if (n == 0) return VG_OK;
  if (!x || !y || !z || !in || !order) return fail(VG_EINVAL, "null input/output array");
  if (n > 0xffffffffull) return fail(VG_EINVAL, "more than 2^32-1 tracks in one call");
  const size_t need = vg::nav_sort_workspace_bytes(n);
  if (!workspace || workspace_bytes < need || (reinterpret_cast<uintptr_t>(workspace) & 255u))
    return fail(VG_EINVAL, "workspace missing, too small or not 256-byte aligned");
  cudaStream_t s        = (cudaStream_t)stream;
  const uint32_t *sorted = nullptr;
  cudaError_t e = vg::launch_nav_sort(g->geo.dev, g->sort, x, y, z, reinterpret_cast<const vg::NavState *>(in), n,
                                      workspace, &sorted, s);
  if (e != cudaSuccess) return cuda_fail(e, "track sort launch");
  e = cudaMemcpyAsync(order, sorted, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && keys) {
    // the sorted keys sit in the key buffer paired with the final value buffer
    const uint32_t *sk = vg::nav_sort_keys_of(sorted, workspace, n);
    e = cudaMemcpyAsync(keys, sk, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
  }
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "order copy");
}

int vg_nav_set_tuning(vg_geom *g, int32_t cell_bits, int32_t queue_blocks_per_sm)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  if (g->geo.world < 0) return fail(VG_ESTATE, "geometry has no world volume");
  if (cell_bits < 0 || cell_bits > 10) return fail(VG_EINVAL, "cell_bits must be in [0, 10]");
  if (queue_blocks_per_sm < 0 || queue_blocks_per_sm > 8) return fail(VG_EINVAL, "queue_blocks_per_sm must be in [0, 8]");
  g->sort         = sort_params(g->geo, cell_bits);
  g->queue_blocks = queue_blocks_per_sm ? queue_blocks_per_sm : 1;
  return VG_OK;
}

int vg_nav_sort_key_params(const vg_geom *g, float lo[3], float scale[3], int32_t *cell_bits, int32_t *lv_bits)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  if (g->geo.world < 0) return fail(VG_ESTATE, "geometry has no world volume");
  for (int k = 0; k < 3; ++k) {
    if (lo) lo[k] = g->sort.lo[k];
    if (scale) scale[k] = g->sort.scale[k];
  }
  if (cell_bits) *cell_bits = g->sort.cell_bits;
  if (lv_bits) *lv_bits = g->sort.lv_bits;
  return VG_OK;
}

int vg_nav_compute_step_and_next_volume_noalloc(const vg_geom *g, const double *x, const double *y, const double *z,
                                                const double *dx, const double *dy, const double *dz,
                                                const double *step_limit, const vg_navstate *in, vg_navstate *out,
                                                double *step, int32_t *status, size_t n, uint32_t flags,
                                                void *stream)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  if (g->geo.world < 0) return fail(VG_ESTATE, "geometry has no world volume");
  if (n > vg::noalloc_max_tracks())
    return fail(VG_EINVAL, "n = " + std::to_string(n) + " exceeds the fixed scratch capacity of " +
                               std::to_string(vg::noalloc_max_tracks()) + " tracks of the no-allocation entry point");
  if (n > 0 && (!x || !y || !z || !dx || !dy || !dz || !in || !out || !step))
    return fail(VG_EINVAL, "null input/output array");
  void *ws     = nullptr;
  size_t bytes = 0;
  if (step_workspace_bytes(n, flags & kNavFlags) > 0) {
    const cudaError_t e = vg::noalloc_scratch(&ws, &bytes);
    if (e != cudaSuccess) return cuda_fail(e, "no-allocation scratch lookup");
    // the fixed array must hold the workspace of the largest call with every flag
    if (bytes < step_workspace_bytes(vg::noalloc_max_tracks(), kNavFlags))
      return fail(VG_ESTATE, "no-allocation scratch smaller than the workspace of " +
                                 std::to_string(vg::noalloc_max_tracks()) + " tracks");
  }
  vg::StepArgs a{x,   y,   z,   dx,  dy,  dz, step_limit, reinterpret_cast<const vg::NavState *>(in),
                 reinterpret_cast<vg::NavState *>(out), step, status, nullptr, n};
  return step_launch(g, a, flags, ws, bytes, (cudaStream_t)stream);
}

int vg_nav_compute_step_and_safety(const vg_geom *g, const double *x, const double *y, const double *z,
                                   const double *dx, const double *dy, const double *dz, const double *step_limit,
                                   const vg_navstate *in, vg_navstate *out, double *step, double *safety,
                                   int32_t *status, size_t n, uint32_t flags, void *stream)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  if (g->geo.world < 0) return fail(VG_ESTATE, "geometry has no world volume");
  if (flags > VG_PREC_MIXED) return fail(VG_EINVAL, "invalid precision flags");
  if (n > 0 && (!x || !y || !z || !dx || !dy || !dz || !in || !out || !step || !safety))
    return fail(VG_EINVAL, "null input/output array");
  vg::StepArgs a{x,   y,   z,   dx,  dy,  dz, step_limit, reinterpret_cast<const vg::NavState *>(in),
                 reinterpret_cast<vg::NavState *>(out), step, status, nullptr, n};
  const cudaError_t e = vg::launch_step_safety(g->geo.dev, a, safety, flags & VG_PREC_MIXED, (cudaStream_t)stream);
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "step-and-safety launch");
}

int vg_nav_compute_step_and_next_volume_host(vg_geom *g, const double *x, const double *y, const double *z,
                                             const double *dx, const double *dy, const double *dz,
                                             const double *step_limit, const vg_navstate *in, vg_navstate *out,
                                             double *step, int32_t *status, size_t n, uint32_t flags, void *stream)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  if (n == 0) return VG_OK;
  if (!x || !y || !z || !dx || !dy || !dz || !in || !out || !step) return fail(VG_EINVAL, "null input/output array");
  if (flags & ~kNavFlags) return fail(VG_EINVAL, "invalid navigation flags");
  std::lock_guard<std::mutex> lock(g->staging_mutex);
  const size_t nd = n * sizeof(double), ns = n * sizeof(vg_navstate), ni = n * sizeof(int32_t);
  const size_t wsb  = step_workspace_bytes(n, flags);
  const size_t need = 8 * nd + 2 * ns + ni + wsb + 16 * 256;
  if (g->staging_size < need) {
    if (g->staging) cudaFree(g->staging);
    g->staging      = nullptr;
    g->staging_size = 0;
    const cudaError_t e = cudaMalloc(&g->staging, need);
    if (e != cudaSuccess) return cuda_fail(e, "staging allocation");
    g->staging_size = need;
  }
  unsigned char *p = static_cast<unsigned char *>(g->staging);
  size_t off       = 0;
  auto take = [&](size_t bytes) {
    void *q = p + off;
    off += (bytes + 255) & ~size_t(255);
    return q;
  };
  double *d[8];
  for (int k = 0; k < 8; ++k) d[k] = static_cast<double *>(take(nd));
  vg_navstate *din  = static_cast<vg_navstate *>(take(ns));
  vg_navstate *dout = static_cast<vg_navstate *>(take(ns));
  int32_t *dst      = static_cast<int32_t *>(take(ni));
  void *dws         = wsb ? take(wsb) : nullptr;
  cudaStream_t s    = (cudaStream_t)stream;
  const double *src[7] = {x, y, z, dx, dy, dz, step_limit};
  cudaError_t e        = cudaSuccess;
  vg::StepArgs a{d[0], d[1], d[2], d[3], d[4], d[5], step_limit ? d[6] : nullptr,
                 reinterpret_cast<const vg::NavState *>(din), reinterpret_cast<vg::NavState *>(dout), d[7],
                 status ? dst : nullptr, nullptr, n};
  // Sorted schedules: the inputs go over in chunks on a copy stream, and the sort keys (and
  // proposals) of each chunk start as soon as it has arrived, so most of the copy hides
  // behind that work; the radix passes and the step wait for all chunks.
  const bool pipelined = (flags & VG_NAV_SORT) && n >= (size_t(1) << 18);
  if (pipelined) {
    if (!g->copy_stream) {
      e = cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking);
      for (int c = 0; c < vg_geom::kCopyChunks && e == cudaSuccess; ++c)
        e = cudaEventCreateWithFlags(&g->chunk_ready[c], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->steps_ready, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->steps_copied, cudaEventDisableTiming);
      if (e != cudaSuccess) return cuda_fail(e, "copy stream setup");
    }
    const StepWs w = step_ws(dws, n, flags);
    const size_t per = (n + vg_geom::kCopyChunks - 1) / vg_geom::kCopyChunks;
    for (int c = 0; c < vg_geom::kCopyChunks && e == cudaSuccess; ++c) {
      const size_t b = std::min(n, c * per), m = std::min(n, b + per) - b;
      for (int k = 0; k < 7 && e == cudaSuccess; ++k)
        if (src[k] && m) e = cudaMemcpyAsync(d[k] + b, src[k] + b, m * sizeof(double), cudaMemcpyHostToDevice, g->copy_stream);
      if (e == cudaSuccess && m)
        e = cudaMemcpyAsync(din + b, in + b, m * sizeof(vg_navstate), cudaMemcpyHostToDevice, g->copy_stream);
      if (e == cudaSuccess) e = cudaEventRecord(g->chunk_ready[c], g->copy_stream);
    }
    if (e != cudaSuccess) return cuda_fail(e, "host-to-device copy");
    for (int c = 0; c < vg_geom::kCopyChunks && e == cudaSuccess; ++c) {
      const size_t b = std::min(n, c * per), m = std::min(n, b + per) - b;
      e = cudaStreamWaitEvent(s, g->chunk_ready[c], 0);
      if (e == cudaSuccess)
        e = vg::launch_nav_sort_keys(g->geo.dev, g->sort, a.x, a.y, a.z, a.in, b, b + m, w.sort, s);
      if (e == cudaSuccess && (flags & VG_NAV_LEARNED) && m) {
        vg::StepArgs pa{a.x + b, a.y + b, a.z + b, a.dx + b, a.dy + b, a.dz + b, nullptr, a.in + b,
                        nullptr,  nullptr, nullptr, nullptr, m};
        e = propose_launch(g, pa, w.slots + b, s);
      }
    }
    if (e != cudaSuccess) return cuda_fail(e, "key/proposal launch");
  } else {
    for (int k = 0; k < 7 && e == cudaSuccess; ++k)
      if (src[k]) e = cudaMemcpyAsync(d[k], src[k], nd, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(din, in, ns, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "host-to-device copy");
  }
  // With the work queue the launcher records steps_ready once the step lengths are final
  // (before a split step's relocation kernel), so they travel back on the copy stream while
  // the relocation still runs; the out-states follow the whole step.
  const bool early_steps = pipelined && (flags & VG_NAV_QUEUE);
  if (early_steps) a.steps_done = g->steps_ready;
  const int rc = step_launch(g, a, flags, dws, wsb, s, pipelined);
  if (rc != VG_OK) return rc;
  if (early_steps) {
    e = cudaStreamWaitEvent(g->copy_stream, g->steps_ready, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(step, d[7], nd, cudaMemcpyDeviceToHost, g->copy_stream);
    if (e == cudaSuccess) e = cudaEventRecord(g->steps_copied, g->copy_stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, ns, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, g->steps_copied, 0);
  } else {
    e = cudaMemcpyAsync(out, dout, ns, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(step, d[7], nd, cudaMemcpyDeviceToHost, s);
  }
  if (e == cudaSuccess && status) e = cudaMemcpyAsync(status, dst, ni, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "device-to-host copy");
}


int vg_mlp_create(const vg_geom *g, uint64_t seed, vg_mlp **out)
{
  if (!out) return fail(VG_EINVAL, "null output handle");
  *out = nullptr;
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  vg_mlp *m = new (std::nothrow) vg_mlp;
  if (!m) return fail(VG_ENOMEM, "out of host memory");
  m->n_lv    = (int)g->geo.lvs.size();
  m->nparams = vg::mlp_param_count(m->n_lv);
  std::vector<float> h(m->nparams, 0.f);
  std::mt19937_64 rng(seed);
  auto fill = [&](int off, int n, float lim) {
    std::uniform_real_distribution<float> u(-lim, lim);
    for (int i = 0; i < n; ++i) h[off + i] = u(rng);
  };
  fill(vg::kMlpW1, vg::kMlpHid * vg::kMlpIn, std::sqrt(6.f / vg::kMlpIn));
  fill(vg::kMlpW2, vg::kMlpHid * vg::kMlpHid, std::sqrt(6.f / vg::kMlpHid));
  fill(vg::kMlpW3, vg::kMlpOut * vg::kMlpHid, std::sqrt(6.f / vg::kMlpHid));
  fill(vg::kMlpE, m->n_lv * vg::kMlpEmb, 0.1f);
  const size_t P = m->nparams;
  cudaError_t e  = cudaMalloc(&m->params, P * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->grads, P * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->m, P * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->v, P * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->wbf, P * sizeof(uint16_t));
  if (e == cudaSuccess) e = cudaMalloc(&m->err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(m->err, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(m->m, 0, P * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(m->v, 0, P * sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(m->params, h.data(), P * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = vg::launch_mlp_to_bf16(m->params, m->wbf, P, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    delete m;
    return cuda_fail(e, "model allocation");
  }
  *out = m;
  return VG_OK;
}

void vg_mlp_destroy(vg_mlp *m) { delete m; }

size_t vg_mlp_param_count(const vg_mlp *m) { return m ? m->nparams : 0; }

int vg_mlp_get_params(const vg_mlp *m, float *host, size_t n)
{
  if (!m || !host || n < m->nparams) return fail(VG_EINVAL, "null model/output or buffer too small");
  const cudaError_t e = cudaMemcpy(host, m->params, m->nparams * sizeof(float), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "parameter copy");
}

int vg_mlp_set_params(vg_mlp *m, const float *host, size_t n)
{
  if (!m || !host || n != m->nparams) return fail(VG_EINVAL, "null model/input or wrong parameter count");
  cudaError_t e = cudaMemcpy(m->params, host, n * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->m, 0, n * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(m->v, 0, n * sizeof(float));
  if (e == cudaSuccess) e = vg::launch_mlp_to_bf16(m->params, m->wbf, n, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  m->t = 0;
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "parameter upload");
}

int vg_learn_features(const vg_geom *g, const double *x, const double *y, const double *z, const double *dx,
                      const double *dy, const double *dz, const vg_navstate *in, size_t n, float *feat, int32_t *lv,
                      int8_t *label, void *stream)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  if (n > 0 && (!x || !y || !z || !dx || !dy || !dz || !in || !feat || !lv))
    return fail(VG_EINVAL, "null input/output array");
  vg::StepArgs a{x, y, z, dx, dy, dz, nullptr, reinterpret_cast<const vg::NavState *>(in), nullptr, nullptr, nullptr,
                 nullptr, n};
  const cudaError_t e = vg::launch_learn_features(g->geo.dev, a, feat, lv, label, (cudaStream_t)stream);
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "feature kernel launch");
}

int vg_mlp_gradients(vg_mlp *m, const float *feat, const int32_t *lv, const int8_t *label, size_t n, float *grads,
                     float *loss, void *stream)
{
  if (!m || !feat || !lv || !label || !grads || !loss) return fail(VG_EINVAL, "null argument");
  if (n == 0 || n > (1u << 24)) return fail(VG_EINVAL, "n must be in [1, 2^24]");
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e  = grow(m->ws, m->ws_floats, vg::mlp_train_ws_floats((int)n));
  if (e == cudaSuccess) e = grow(m->idx, m->idx_n, n);
  if (e != cudaSuccess) return cuda_fail(e, "scratch allocation");
  std::vector<uint32_t> id(n);
  for (size_t i = 0; i < n; ++i) id[i] = (uint32_t)i;
  e = cudaMemcpyAsync(m->idx, id.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = vg::launch_mlp_grad(m->params, m->n_lv, feat, lv, label, m->idx, (int)n, grads, loss, m->ws, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "gradient kernels");
}

int vg_mlp_train(vg_mlp *m, const float *feat, const int32_t *lv, const int8_t *label, size_t n, int32_t epochs,
                 int32_t batch, float lr, uint64_t seed, float *epoch_loss, void *stream)
{
  if (!m || !feat || !lv || !label) return fail(VG_EINVAL, "null argument");
  if (n == 0 || n > 0xffffffffull || epochs < 0 || batch < 1 || batch > 65536 || !(lr > 0))
    return fail(VG_EINVAL, "invalid training parameters");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t nbatch = (n + batch - 1) / batch;
  size_t loss_cap     = 0;
  float *losses       = nullptr;
  cudaError_t e       = grow(m->ws, m->ws_floats, vg::mlp_train_ws_floats(batch));
  if (e == cudaSuccess) e = grow(m->idx, m->idx_n, n);
  if (e == cudaSuccess) e = grow(losses, loss_cap, nbatch);
  if (e != cudaSuccess) {
    if (losses) cudaFree(losses);
    return cuda_fail(e, "scratch allocation");
  }
  std::vector<uint32_t> perm(n);
  std::vector<float> hl(nbatch);
  std::mt19937_64 rng(seed);
  for (int ep = 0; ep < epochs && e == cudaSuccess; ++ep) {
    for (size_t i = 0; i < n; ++i) perm[i] = (uint32_t)i;
    std::shuffle(perm.begin(), perm.end(), rng);
    e = cudaMemcpyAsync(m->idx, perm.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    for (size_t b = 0; b < nbatch && e == cudaSuccess; ++b) {
      const size_t b0 = b * batch;
      const int nb    = (int)std::min<size_t>(batch, n - b0);
      e = vg::launch_mlp_grad(m->params, m->n_lv, feat, lv, label, m->idx + b0, nb, m->grads, losses + b, m->ws, s);
      if (e == cudaSuccess)
        e = vg::launch_mlp_adam(m->params, m->grads, m->m, m->v, m->nparams, lr, 0.9f, 0.999f, 1e-8f, ++m->t, s);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hl.data(), losses, nbatch * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && epoch_loss) {
      double sum = 0.;
      for (float v : hl) sum += v;
      epoch_loss[ep] = (float)(sum / (double)n);
    }
  }
  if (e == cudaSuccess) e = vg::launch_mlp_to_bf16(m->params, m->wbf, m->nparams, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(losses);
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "training");
}

int vg_mlp_infer(const vg_mlp *m, const float *feat, const int32_t *lv, size_t n, int8_t *slot, float *logits,
                 uint32_t flags, void *stream)
{
  if (!m || (n > 0 && (!feat || !lv || !slot))) return fail(VG_EINVAL, "null argument");
  if (flags > 1) return fail(VG_EINVAL, "unknown inference flags");
  const cudaError_t e =
      flags ? vg::launch_mlp_infer_feat_tc(m->wbf, feat, lv, n, slot, logits, m->err, (cudaStream_t)stream)
            : vg::launch_mlp_infer_feat(m->wbf, m->n_lv, feat, lv, n, slot, logits, (cudaStream_t)stream);
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "inference kernel launch");
}

int vg_nav_propose(const vg_geom *g, const double *x, const double *y, const double *z, const double *dx,
                   const double *dy, const double *dz, const vg_navstate *in, size_t n, int8_t *slot, uint32_t flags,
                   void *stream)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  if (!g->proposer) return fail(VG_ESTATE, "no proposer model attached");
  if (flags > 1) return fail(VG_EINVAL, "unknown proposal flags");
  if (n > 0 && (!x || !y || !z || !dx || !dy || !dz || !in || !slot)) return fail(VG_EINVAL, "null input/output array");
  vg::StepArgs a{x, y, z, dx, dy, dz, nullptr, reinterpret_cast<const vg::NavState *>(in), nullptr, nullptr, nullptr,
                 nullptr, n};
  const cudaError_t e =
      flags ? vg::launch_mlp_propose_tc(g->geo.dev, a, g->proposer->wbf, slot, g->proposer->err, (cudaStream_t)stream)
            : vg::launch_mlp_propose(g->geo.dev, a, g->proposer->wbf, slot, (cudaStream_t)stream);
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "proposal launch");
}

int vg_nav_set_proposal_kernel(vg_geom *g, int32_t tensor)
{
  if (!g) return fail(VG_EINVAL, "null geometry handle");
  g->propose_tensor = tensor ? 1 : 0;
  return VG_OK;
}

int vg_mlp_error(const vg_mlp *m, int32_t *error)
{
  if (!m || !error) return fail(VG_EINVAL, "null argument");
  int h = 0;
  cudaError_t e = cudaMemcpy(&h, m->err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(m->err, 0, sizeof(int));
  *error = h;
  return e == cudaSuccess ? VG_OK : cuda_fail(e, "error flag read");
}

int vg_geom_set_proposer(vg_geom *g, const vg_mlp *m)
{
  if (!closed_ok(g)) return g ? VG_ESTATE : VG_EINVAL;
  if (m && m->n_lv != (int)g->geo.lvs.size()) return fail(VG_EINVAL, "model was made for another geometry");
  g->proposer = m;
  return VG_OK;
}

} // extern "C"

// SoA shape-query kernels (one instantiation per shape type and query, the shape record
// passed by value so every lane reads it from the constant bank). Compiled with
// --fmad=false; FP64 compares and min/max run on the integer pipe (VG_FP64_INT_COMPARE,
// fp64_int.cuh), which these throughput-bound kernels gain from.
#include "launch.h"
#include "nav_fp64.cuh"
#include "shapes_mixed.cuh"
#include "shapes_poly_mixed.cuh"
#include <type_traits>

namespace vg {
namespace {

using f64::V3;

// Grid: enough CTAs to fill the 152 SMs several times over, then grid-stride.
inline unsigned grid_for(size_t n, int block)
{
  size_t blocks       = (n + block - 1) / block;
  const size_t maxgrd = 152 * 16;
  if (blocks > maxgrd) blocks = maxgrd;
  return (unsigned)(blocks ? blocks : 1);
}

template <class R>
struct ShapeOps;
#define VG_OPS(R, PFX)                                                                              \
  template <>                                                                                       \
  struct ShapeOps<R> {                                                                              \
    __device__ static int inside(const R &r, V3 p) { return f64::PFX##_inside(r, p); }              \
    __device__ static bool contains(const R &r, V3 p) { return f64::PFX##_contains(r, p); }         \
    __device__ static double dist_in(const R &r, V3 p, V3 d) { return f64::PFX##_dist_in(r, p, d); }   \
    __device__ static double dist_out(const R &r, V3 p, V3 d) { return f64::PFX##_dist_out(r, p, d); } \
    __device__ static double safety_in(const R &r, V3 p) { return f64::PFX##_safety_in(r, p); }     \
    __device__ static double safety_out(const R &r, V3 p) { return f64::PFX##_safety_out(r, p); }   \
  };
VG_OPS(BoxRec, box)
VG_OPS(TubeRec, tube)
VG_OPS(ConeRec, cone)
VG_OPS(TrdRec, trd)
VG_OPS(TrapRec, trap)
VG_OPS(TorusRec, torus)
VG_OPS(CutTubeRec, cuttube)
VG_OPS(SphereRec, sphere)
VG_OPS(GenTrapRec, gentrap)
VG_OPS(HypeRec, hype)
#undef VG_OPS

// Q: 0 Inside, 1 Contains, 2 DistanceToIn, 3 DistanceToOut, 4 SafetyToIn, 5 SafetyToOut.
// M: mixed precision (FP32 guard on the descriptor `lb`, see shapes_mixed.cuh).
template <class R, int Q, bool M>
__global__ void __launch_bounds__(256) k_shape_query(const R rec, const Xform xf, const int apply_xf,
                                                     const mixed::ShapeLB lb, const double *__restrict__ x,
                                                     const double *__restrict__ y, const double *__restrict__ z,
                                                     const double *__restrict__ dx, const double *__restrict__ dy,
                                                     const double *__restrict__ dz, size_t n, void *__restrict__ out)
{
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    V3 p{__ldg(x + i), __ldg(y + i), __ldg(z + i)};
    const bool framed = apply_xf && (Q == 0 || Q == 1 || Q == 2 || Q == 4);
    if (framed) p = f64::to_local(xf, p);
    if (Q == 0 || Q == 1) {
      const int c = M ? mixed::lb_classify(lb, p) : 0;
      if (Q == 0) static_cast<int32_t *>(out)[i] = c ? c : ShapeOps<R>::inside(rec, p);
      if (Q == 1) static_cast<uint8_t *>(out)[i] = c ? (c == kInside ? 1 : 0) : (ShapeOps<R>::contains(rec, p) ? 1 : 0);
    }
    if (Q == 2 || Q == 3) {
      V3 d{__ldg(dx + i), __ldg(dy + i), __ldg(dz + i)};
      if (framed) d = f64::rotate(xf, d);
      double r;
      if (Q == 2)
        r = (M && mixed::lb_certain_miss(lb, p, d)) ? kInfLength : ShapeOps<R>::dist_in(rec, p, d);
      else
        r = ShapeOps<R>::dist_out(rec, p, d);
      static_cast<double *>(out)[i] = r;
    }
    if (Q == 4 || Q == 5) {
      double r;
      if (M && std::is_same<R, TubeRec>::value && !f64::tube_phi(reinterpret_cast<const TubeRec &>(rec)) &&
               mixed::in_range(mixed::f3(p)))
        r = mixed::tube_safety_mixed(reinterpret_cast<const TubeRec &>(rec), p, Q == 5);
      else
        r = (Q == 4) ? ShapeOps<R>::safety_in(rec, p) : ShapeOps<R>::safety_out(rec, p);
      static_cast<double *>(out)[i] = r;
    }
  }
}

// Mixed-precision SoA distance query with block-level compaction. Each thread first tries to
// settle its query in FP32 (exact-shape classification with a kBoxPad margin, certain misses of the
// padded descriptor; see shapes_mixed.cuh). Queries it cannot settle go to a shared-memory
// queue, and whenever the queue holds a full block's worth, all 256
// threads evaluate 256 of them in FP64, so the FP64 code runs with full warps instead of the
// few lanes that needed it. Results are those of the FP64 kernel (k_shape_query<R, Q,
// false>) for every query.
template <class R, int Q>
__global__ void __launch_bounds__(256) k_shape_query_mixed(const R rec, const Xform xf, const int apply_xf,
                                                           const mixed::ShapeLB lb, const double *__restrict__ x,
                                                           const double *__restrict__ y, const double *__restrict__ z,
                                                           const double *__restrict__ dx, const double *__restrict__ dy,
                                                           const double *__restrict__ dz, size_t n,
                                                           void *__restrict__ out)
{
  __shared__ unsigned long long queue[512];
  __shared__ int qn;
  if (threadIdx.x == 0) qn = 0;
  __syncthreads();
  static_assert(Q == 2 || Q == 3, "distances only");
  const bool framed = apply_xf && Q == 2;
  // FP32 frame: p - t in FP32 (|p|, |t| <= kMaxCoord keep it within 1e-3 mm), FP32 rotation
  const bool ident = f64::rot_is_identity(xf);
  const float tf[3] = {(float)xf.t[0], (float)xf.t[1], (float)xf.t[2]};
  const bool t_ok   = mixed::in_range(mixed::F3{tf[0], tf[1], tf[2]});
  auto local_f = [&](mixed::F3 v, bool point) {
    if (!framed) return v;
    if (point) v = mixed::F3{v.x - tf[0], v.y - tf[1], v.z - tf[2]};
    if (ident) return v;
    return mixed::F3{fmaf(v.x, (float)xf.r[0], fmaf(v.y, (float)xf.r[3], v.z * (float)xf.r[6])),
                     fmaf(v.x, (float)xf.r[1], fmaf(v.y, (float)xf.r[4], v.z * (float)xf.r[7])),
                     fmaf(v.x, (float)xf.r[2], fmaf(v.y, (float)xf.r[5], v.z * (float)xf.r[8]))};
  };
  auto fast = [&](size_t i) -> bool {
    const mixed::F3 pg{(float)__ldg(x + i), (float)__ldg(y + i), (float)__ldg(z + i)};
    if (!mixed::in_range(pg) || (framed && !t_ok)) return false;
    const mixed::F3 l = local_f(pg, true);
    const int c       = mixed::f32_classify(rec, lb, l);
    if (Q == 2) {
      if (c == kInside && mixed::dist_in_inside_is_minus1<R>()) {
        static_cast<double *>(out)[i] = -1.0;
        return true;
      }
      if (c != kOutside) return false;
      const mixed::F3 d = local_f(mixed::F3{(float)__ldg(dx + i), (float)__ldg(dy + i), (float)__ldg(dz + i)}, false);
      if (!mixed::f32_certain_miss(lb, l, d)) return false;
      static_cast<double *>(out)[i] = kInfLength;
      return true;
    }
    if (Q == 3 && c == kOutside && mixed::dist_out_outside_is_minus1(rec)) {
      static_cast<double *>(out)[i] = -1.0;
      return true;
    }
    return false;
  };
  auto exact = [&](size_t i) {
    V3 p{__ldg(x + i), __ldg(y + i), __ldg(z + i)};
    V3 d{__ldg(dx + i), __ldg(dy + i), __ldg(dz + i)};
    if (framed) p = f64::to_local(xf, p), d = f64::rotate(xf, d);
    static_cast<double *>(out)[i] = (Q == 2) ? ShapeOps<R>::dist_in(rec, p, d) : ShapeOps<R>::dist_out(rec, p, d);
  };
  const int lane      = threadIdx.x & 31;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t base = (size_t)blockIdx.x * blockDim.x; base < n; base += stride) { // uniform over the block
    const size_t i    = base + threadIdx.x;
    const bool undec  = i < n && !fast(i);
    const unsigned bl = __ballot_sync(0xffffffffu, undec);
    if (bl) {
      int w = 0;
      if (lane == 0) w = atomicAdd(&qn, __popc(bl));
      w = __shfl_sync(0xffffffffu, w, 0);
      if (undec) queue[w + __popc(bl & ((1u << lane) - 1u))] = i;
    }
    __syncthreads();
    const int q = qn; // < 512: at most 255 left over plus 256 new
    if (q >= 256) {
      exact(queue[q - 256 + threadIdx.x]);
      __syncthreads();
      if (threadIdx.x == 0) qn = q - 256;
    }
    __syncthreads();
  }
  const int q = qn;
  if ((int)threadIdx.x < q) exact(queue[threadIdx.x]);
}

template <class R, bool M>
cudaError_t launch_typed_q(const R &rec, const Xform &xf, int apply_xf, const mixed::ShapeLB &lb, int q,
                           const QueryArgs &a, cudaStream_t s)
{
  const int block     = 256;
  const unsigned grid = grid_for(a.n, block);
#define VG_Q(Q)                                                                                                   \
  k_shape_query<R, Q, (M && Q >= 4)><<<grid, block, 0, s>>>(rec, xf, apply_xf, lb, a.x, a.y, a.z, a.dx, a.dy, a.dz, \
                                                             a.n, a.out)
#define VG_QM(Q)                                                                                                  \
  (M ? k_shape_query_mixed<R, Q><<<grid, block, 0, s>>>(rec, xf, apply_xf, lb, a.x, a.y, a.z, a.dx, a.dy, a.dz, a.n, \
                                                       a.out)                                                      \
     : k_shape_query<R, Q, false><<<grid, block, 0, s>>>(rec, xf, apply_xf, lb, a.x, a.y, a.z, a.dx, a.dy, a.dz,   \
                                                         a.n, a.out))
  // Inside and Contains are cheaper in the FP64 kernel (integer-pipe compares) than any FP32
  // pre-classification measured (0.7-0.95x of it), so VG_PREC_MIXED uses it for them.
  switch (q) {
  case 0: VG_Q(0); break;
  case 1: VG_Q(1); break;
  case 2: VG_QM(2); break;
  case 3: VG_QM(3); break;
  case 4: VG_Q(4); break;
  case 5: VG_Q(5); break;
  default: return cudaErrorInvalidValue;
  }
#undef VG_Q
#undef VG_QM
  return cudaGetLastError();
}

template <class R>
cudaError_t launch_typed(const double *recp, const Xform &xf, int apply_xf, const float *lbd, int q,
                         const QueryArgs &a, cudaStream_t s)
{
  R rec;
  memcpy(&rec, recp, sizeof(R));
  if (!lbd) return launch_typed_q<R, false>(rec, xf, apply_xf, mixed::ShapeLB{}, q, a, s);
  mixed::ShapeLB lb;
  memcpy(&lb, lbd, sizeof(lb));
  return launch_typed_q<R, true>(rec, xf, apply_xf, lb, q, a, s);
}

// Variable-length and composite shapes (polycone, polyhedron, boolean): the record stays in
// the geometry arena and the query goes through the run-time dispatch.
template <int Q, bool M>
__global__ void __launch_bounds__(256) k_shape_query_dyn(const DevGeom g, const int shape, const Xform xf,
                                                         const int apply_xf, const double *__restrict__ x,
                                                         const double *__restrict__ y,
                                                         const double *__restrict__ z, const double *__restrict__ dx,
                                                         const double *__restrict__ dy, const double *__restrict__ dz,
                                                         size_t n, void *__restrict__ out)
{
  const mixed::ShapeLB lb = M ? reinterpret_cast<const mixed::ShapeLB *>(g.shape_lbd)[shape] : mixed::ShapeLB{};
  const bool poly         = g.shape_type[shape] == kShapePolyhedron;
  const bool pcone        = g.shape_type[shape] == kShapePolycone;
  const int off           = g.shape_off[shape];
  const size_t stride     = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    V3 p{__ldg(x + i), __ldg(y + i), __ldg(z + i)};
    const bool framed = apply_xf && (Q == 0 || Q == 1 || Q == 2 || Q == 4);
    if (framed) p = f64::to_local(xf, p);
    if (Q == 0 || Q == 1) {
      const int c = M ? mixed::lb_classify(lb, p) : 0;
      if (Q == 0) static_cast<int32_t *>(out)[i] = c ? c : f64::shape_inside(g, shape, p);
      if (Q == 1)
        static_cast<uint8_t *>(out)[i] = c ? (c == kInside ? 1 : 0) : (f64::shape_contains(g, shape, p) ? 1 : 0);
    }
    if (Q == 2 || Q == 3) {
      V3 d{__ldg(dx + i), __ldg(dy + i), __ldg(dz + i)};
      if (framed) d = f64::rotate(xf, d);
      double r;
      if (M && poly) { // FP32-screened quadrilaterals, same FP64 results
        const PolyhedronRec &rec = f64::rec_at<PolyhedronRec>(g, off);
        r = (Q == 2) ? (mixed::lb_certain_miss(lb, p, d) ? kInfLength : mixed::polyhedron_dist_in_mixed(rec, p, d))
                     : mixed::polyhedron_dist_out_mixed(rec, p, d);
      } else if (M && pcone && Q == 2) { // FP32-screened sections, same FP64 results
        r = mixed::lb_certain_miss(lb, p, d) ? kInfLength
                                             : mixed::polycone_dist_in_mixed(f64::rec_at<PolyconeRec>(g, off), p, d);
      } else {
        r = (Q == 2) ? ((M && mixed::lb_certain_miss(lb, p, d)) ? kInfLength : f64::shape_dist_in(g, shape, p, d))
                     : f64::shape_dist_out(g, shape, p, d);
      }
      static_cast<double *>(out)[i] = r;
    }
    if (Q == 4) static_cast<double *>(out)[i] = f64::shape_safety_in(g, shape, p);
    if (Q == 5) static_cast<double *>(out)[i] = f64::shape_safety_out(g, shape, p);
  }
}

// Polycone DistanceToOut with lane refill. The section loop of PolyconeImplementation.h
// runs 1 to nsec passes per ray, so in the plain kernel a warp waits for its longest ray.
// Here each lane walks its own grid-stride sequence of queries: every round, a lane without
// a query in progress sets up its next one (which may end at once), and every lane with a
// section loop in progress runs one pass of it. The passes of a round run together, and a
// lane whose ray is done starts the next instead of idling. Each query runs the same setup
// and passes as polycone_dist_out, so the results are its results.
__global__ void __launch_bounds__(256) k_polycone_dist_out_refill(const DevGeom g, const int shape,
                                                                  const double *__restrict__ x,
                                                                  const double *__restrict__ y,
                                                                  const double *__restrict__ z,
                                                                  const double *__restrict__ dx,
                                                                  const double *__restrict__ dy,
                                                                  const double *__restrict__ dz, size_t n,
                                                                  double *__restrict__ out)
{
  const f64::PolyconeView v(f64::rec_at<PolyconeRec>(g, g.shape_off[shape]));
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i            = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  f64::PolyconeOutLoop L;
  bool busy = false;
  for (;;) {
    double r;
    if (!busy && i < n) {
      if (f64::polycone_out_setup(v, V3{__ldg(x + i), __ldg(y + i), __ldg(z + i)},
                                  V3{__ldg(dx + i), __ldg(dy + i), __ldg(dz + i)}, r, L)) {
        out[i] = r;
        i += stride;
      } else {
        busy = true;
      }
    }
    if (busy && f64::polycone_out_pass(v, L, r)) {
      out[i] = r;
      i += stride;
      busy = false;
    }
    if (!__any_sync(0xffffffffu, busy || i < n)) break;
  }
}

} // namespace

cudaError_t launch_shape_query_fp64(int type, const double *rec, const Xform &xf, int apply_xf, int q,
                                    const QueryArgs &a, cudaStream_t s, const float *lbd)
{
  if (a.n == 0) return cudaSuccess;
  switch (type) {
  case kShapeBox: return launch_typed<BoxRec>(rec, xf, apply_xf, lbd, q, a, s);
  case kShapeTube: return launch_typed<TubeRec>(rec, xf, apply_xf, lbd, q, a, s);
  case kShapeCone: return launch_typed<ConeRec>(rec, xf, apply_xf, lbd, q, a, s);
  case kShapeTrd: return launch_typed<TrdRec>(rec, xf, apply_xf, lbd, q, a, s);
  case kShapeTrap: return launch_typed<TrapRec>(rec, xf, apply_xf, lbd, q, a, s);
  case kShapeTorus2: return launch_typed<TorusRec>(rec, xf, apply_xf, lbd, q, a, s);
  case kShapeCutTube: return launch_typed<CutTubeRec>(rec, xf, apply_xf, lbd, q, a, s);
  case kShapeSphere: return launch_typed<SphereRec>(rec, xf, apply_xf, lbd, q, a, s);
  case kShapeGenTrap: return launch_typed<GenTrapRec>(rec, xf, apply_xf, lbd, q, a, s);
  case kShapeHype: return launch_typed<HypeRec>(rec, xf, apply_xf, lbd, q, a, s);
  default: return cudaErrorNotSupported;
  }
}

cudaError_t launch_shape_query_dyn_fp64(const DevGeom &g, int shape, int type, const Xform &xf, int apply_xf, int q,
                                        const QueryArgs &a, cudaStream_t s, bool mixed)
{
  if (a.n == 0) return cudaSuccess;
  const unsigned grid = grid_for(a.n, 256);
  if (q == 3 && type == kShapePolycone) { // DistanceToOut takes local points: no transform
    k_polycone_dist_out_refill<<<grid, 256, 0, s>>>(g, shape, a.x, a.y, a.z, a.dx, a.dy, a.dz, a.n,
                                                    static_cast<double *>(a.out));
    return cudaGetLastError();
  }
#define VG_DYN(Q)                                                                                                   \
  (mixed ? k_shape_query_dyn<Q, true><<<grid, 256, 0, s>>>(g, shape, xf, apply_xf, a.x, a.y, a.z, a.dx, a.dy, a.dz, \
                                                           a.n, a.out)                                             \
         : k_shape_query_dyn<Q, false><<<grid, 256, 0, s>>>(g, shape, xf, apply_xf, a.x, a.y, a.z, a.dx, a.dy, a.dz, \
                                                            a.n, a.out))
  switch (q) {
  case 0: mixed = false, VG_DYN(0); break; // FP64 is the faster classification (see launch_typed_q)
  case 1: mixed = false, VG_DYN(1); break;
  case 2: VG_DYN(2); break;
  case 3: VG_DYN(3); break;
  case 4: VG_DYN(4); break;
  case 5: VG_DYN(5); break;
  default: return cudaErrorInvalidValue;
  }
#undef VG_DYN
  return cudaGetLastError();
}

} // namespace vg

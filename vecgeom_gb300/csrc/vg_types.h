// Plain-old-data records of the flattened device geometry, shared by the host builder
// (geom.cpp) and the CUDA kernels. One record per unplaced shape, holding the user
// parameters plus every quantity the reference precomputes at construction time
// (VecGeom/volumes/*Struct.h), so no kernel evaluates a transcendental function.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define VG_HD __host__ __device__
#else
#define VG_HD
#endif

namespace vg {

// Shape type tags (also the C-ABI's VG_SHAPE_* values).
enum ShapeType : int32_t {
  kShapeBox        = 1,
  kShapeTube       = 2,
  kShapeCone       = 3,
  kShapePolycone   = 4,
  kShapePolyhedron = 5,
  kShapeTorus2     = 6,
  kShapeTrd        = 7,
  kShapeBoolMinus  = 8,
  kShapeTrap       = 9,
  kShapeCutTube    = 10,
  kShapeSphere     = 11,
  kShapeGenTrap    = 12,
  kShapeHype       = 13,
};

// The navigator's core shape set. Navigation kernels are also compiled with the dispatch of
// these types only (smaller code: fewer instruction-cache misses in the step kernels); the
// host runs that build for a geometry whose shapes all lie in the set (DevGeom::type_mask).
constexpr uint32_t kCoreShapeMask = (1u << kShapeBox) | (1u << kShapeTube) | (1u << kShapeCone) |
                                    (1u << kShapePolycone) | (1u << kShapeTrd);

// VecGeom/base/Math.h:27-52 (double precision)
constexpr double kTolerance     = 1e-9;
constexpr double kHalfTolerance = 0.5 * kTolerance;
constexpr double kConeTolerance = 1e-7;
constexpr double kPushTolerance = 1e-6;
constexpr double kAngTolerance  = 1e-9;
constexpr double kPi            = 3.14159265358979323846;
constexpr double kTwoPi         = 2. * kPi;
constexpr double kInfLength     = 1.7976931348623157e308; // DBL_MAX
constexpr double kEpsilon       = 2.220446049250313e-16;  // DBL_EPSILON
constexpr double kMinimum       = 2.2250738585072014e-308; // DBL_MIN

// EnumInside (VecGeom/base/Global.h:71-79)
constexpr int32_t kInside = 1, kSurface = 2, kOutside = 3;

// Phi wedge (VecGeom/volumes/Wedge_Evolution.h): along and normal vectors of both planes.
struct WedgeRec {
  double dphi;
  double a1x, a1y, a2x, a2y;
  double n1x, n1y, n2x, n2y;
};

struct BoxRec {
  double dx, dy, dz;
};

// VecGeom/volumes/TubeStruct.h:15-41
struct TubeRec {
  double rmin, rmax, z, sphi, dphi;
  double rmin2, rmax2, a1x, a1y, a2x, a2y;
  double tolIrmin2, tolOrmin2, tolIrmax2, tolOrmax2, tolIz, tolOz;
  double tolIrmin, tolOrmin, tolIrmax, tolOrmax, maxVal;
  WedgeRec w;
};

// VecGeom/volumes/ConeStruct.h:23-83
struct ConeRec {
  double rmin1, rmax1, rmin2, rmax2, dz, sphi, dphi;
  double frmin1, frmin2, frmax1, frmax2; // construction values (used by Extent)
  double a1x, a1y, a2x, a2y;
  double innerSlope, outerSlope, innerOffset, outerOffset, innerTol, outerTol;
  double sqRmin1, sqRmin2, sqRmax1, sqRmax2, tolIz, tolOz;
  double innerApex, tanInnerApex, outerApex, tanOuterApex;
  double secRMin, secRMax, invSecRMin, invSecRMax, tanRMin, tanRMax, zNormInner, zNormOuter;
  double origRmax1, origRmax2;
  WedgeRec w;
};

// VecGeom/volumes/TrdStruct.h:15-86
struct TrdRec {
  double dx1, dx2, dy1, dy2, dz;
  double x2minusx1, y2minusy1, halfx1plusx2, halfy1plusy2, calfx, calfy, fx, fy, tolx, toly, pad;
};

// VecGeom/volumes/TrapezoidStruct.h:20-63 in the VECGEOM_PLANESHELL build (PlaneShell<4>,
// VecGeom/base/PlaneShell.h:25-31): half length in z, dz -+ kHalfTolerance, and the four side
// planes a x + b y + c z + d (outward unit normals) in the order -Y, +Y, -X, +X.
struct TrapRec {
  double dz, dz_plus, dz_minus, pad;
  double a[4], b[4], c[4], d[4];
};

// Polycone record: header, section boundaries, then one (shift, cone) block per section
// (VecGeom/volumes/PolyconeStruct.h:26-36, PolyconeSection.h). Variable length; the views
// below address it in place.
// Each section block: z shift, then four FP32 values in the next two doubles (the section's
// conservative cylindrical shell in the polycone frame, padded by 4e-3 mm and rounded
// outward: rmin, rmax, zlo, zhi; for the mixed-precision screen), one pad double, ConeRec.
struct PolyconeRec {
  double nsec, sphi, dphi, reserved;
  double data[1]; // zs[nsec+1], pad to a multiple of 4, then nsec x (shift, shell, pad, ConeRec, pad)
};
constexpr int kPolyconeSectionDoubles = 4 + ((int)(sizeof(ConeRec) / sizeof(double)) + 3) / 4 * 4;
VG_HD inline int polycone_section_base(int nsec) { return ((4 + nsec + 1) + 3) / 4 * 4; }

// VecGeom/volumes/TorusStruct2.h:26-43 (+ the bounding tube of UnplacedTorus2.h:64-74)
struct TorusRec {
  double rmin, rmax, rtor, sphi, dphi, rmin2, rmax2, rtor2;
  WedgeRec w;
  double pad[3];
  TubeRec bt;
};

// Polyhedron record (VecGeom/volumes/PolyhedronStruct.h:52-107): fixed header, then the
// z planes, radii, same-z flags and phi-section normals, a segment table (n_outer, n_phi,
// n_inner, first quadrilateral) and the quadrilaterals of all segments (outer, phi, inner
// in that order), kPolyQuadDoubles each: plane normal + distance, four side planes
// (normal + distance) and four corners (Quadrilaterals.h:28-37). Offsets in doubles from
// the record start. After the quadrilaterals, an FP32 copy of each one's planes (normal +
// distance, then the four side planes: kPolyQuadFloats floats, rounded to nearest) in the
// same order, for the mixed-precision screens: quadrilateral k (counted from offQuad0) has
// its copy at float offset 2 * offQuadF + kPolyQuadFloats * k.
struct PolyhedronRec {
  double nsides, nseg, nz, flags; // flags: 1 inner radii, 2 phi cutout, 4 phi cutout > pi
  double phiStart, phiDelta, tubeOffset, pad0;
  double offZ, offRMin, offRMax, offSameZ, offPhiSec, offSeg, offQuad0, offQuadF;
  WedgeRec w;
  double pad3[3];
  TubeRec bt;
};
constexpr int kPolyQuadDoubles = 32; // n[3] d | (sideN[3] sideD) x 4 | corner[3] x 4
constexpr int kPolyQuadFloats  = 20; // n[3] d | (sideN[3] sideD) x 4
constexpr int kPolyFlagInner = 1, kPolyFlagPhi = 2, kPolyFlagLargePhi = 4;

// Cut tube (VecGeom/volumes/CutTubeStruct.h:22-49): the tube record of UniversalTube with
// infinite half-length, the two cut planes (unit normal and distance, Plane.h:40-49: bottom
// through (0, 0, -dz), top through (0, 0, +dz)), dz and the far-point scale max(rmax, dz).
struct CutTubeRec {
  TubeRec t;
  double n0x, n0y, n0z, d0, n1x, n1y, n1z, d1;
  double dz, maxVal, pad0, pad1;
};

// Sphere (VecGeom/volumes/SphereStruct.h:20-276): radii and the checked angles, the full-
// phi / full-theta flags, the phi wedge and the theta cone (ThetaCone_Evolution.h:21-69)
// made from the constructor's raw angles, as the reference makes them.
struct SphereRec {
  double rmin, rmax, sphi, dphi, stheta, dtheta, eTheta;
  double fullPhi, fullTheta, fullSphere; // 0 or 1
  WedgeRec w;
  double tcS, tcE, tanS, tanE, tanS2, tanE2, tanBis, slope1, slope2, pad0;
};

// Generic trapezoid (VecGeom/volumes/GenTrapStruct.h with its SecondOrderSurfaceShell<4>,
// SecondOrderSurfaceShell.h): the eight vertices in the clockwise order the reference keeps
// (bottom 0-3 at -dz, top 4-7 at +dz), the bounding box, the section terms of the struct
// and the shell's per-surface terms. Surface i runs from vertex i to vertex (i+1)%4 (and
// their tops): fxa = vx[i], fxb = vx[i+4], fxc = vx[j], fxd = vx[j+4].
struct GenTrapRec {
  double bbdim[3], bborig[3];
  double vx[8], vy[8];
  double dz, invDz, halfInvDz, dz2; // dz2 = 0.5 / dz (the shell's fDz2)
  double connx[4], conny[4];        // vx[i] - vx[i+4]
  double deltax[8], deltay[8];      // edge vectors of the bottom (0-3) and top (4-7) polygons
  double tx1[4], ty1[4], tx2[4], ty2[4], t1crosst2[4], deltatx[4], deltaty[4];
  double normal[4][3], viCrossHi0[4][3], viCrossVj[4][3], hi1CrossHi0[4][3];
  long long degenerated; // bit i: edge i collapsed on both bases (struct and shell agree)
  long long curved;      // bit i: surface i is twisted (SecondOrderSurfaceShell fiscurved)
  long long planar;      // no surface twisted (the shell's fisplanar)
  long long pad;
};

// Hyperboloid (VecGeom/volumes/HypeStruct.h:19-80, CalculateCached): radii at z = 0, stereo
// angles, the half-length and the cached squares, end-cap radii and tolerance levels;
// `inner` is InnerSurfaceExists (rmin > 0 or a non-zero inner stereo angle).
struct HypeRec {
  double rmin, rmax, stIn, stOut, dz;
  double tIn, tOut, tIn2, tOut2, rmin2, rmax2, dz2;
  double endInnerRadius2, endOuterRadius2, endInnerRadius, endOuterRadius;
  double zTol, innerTol, outerTol, inner;
};

// Boolean subtraction record (VecGeom/volumes/BooleanStruct.h:19-33): operand placed-volume ids.
struct BoolRec {
  double left_pv, right_pv, reserved0, reserved1;
};
// Bound of the reference's unbounded push loop in DistanceToIn (BooleanImplementation.h:116-146).
constexpr int kBoolMaxPush = 1000;

// Compact placed-volume transformation: p_local = R^T (p - t) with the reference's
// component order (VecGeom/base/Transformation3D.h:640-651).
struct Xform {
  double t[3];
  double r[9];
};

// Navigation state: bit-identical to NavStateIndex (VecGeom/navigation/NavStateIndex.h:39-41).
struct NavState {
  uint32_t navInd;
  uint32_t lastExited;
  uint8_t onBoundary;
  uint8_t pad[3];
};
static_assert(sizeof(NavState) == 12, "NavState layout");

// FP32 BVH node record for the mixed-precision traversal: 32 bytes, 32-byte aligned.
struct alignas(32) NodeF {
  float lo[3];
  float hi[3];
  int32_t nchild; // >= 0: leaf with nchild prims; -1: internal
  int32_t offset; // first prim slot (absolute index into the prim arrays)
};
static_assert(sizeof(NodeF) == 32, "NodeF layout");

// FP32 record of one BVH prim slot for the mixed-precision traversal, in slot order (the
// order leaves reference): the daughter's box, placed volume, FP32 shape descriptor and
// placement, so that a leaf test, a lower/upper distance bound or a Contains pre-test reads
// one 128-byte line instead of a chain of dependent loads (slot -> daughter -> placed
// volume -> logical volume -> shape -> descriptor, and the transform).
struct alignas(16) LeafRec {
  float lo[3], hi[3]; // daughter box rounded outward (FP32)
  int32_t pv;         // placed volume
  int32_t type;       // shape type of the daughter
  float lb[8];        // FP32 bounding descriptor of the daughter's shape (shape_lbd)
  float t[3];         // placement translation rounded to FP32
  int32_t exact_only; // 1: translation beyond the FP32 range of the pruning (FP64 only)
  int32_t pad[2];
  float r[9];         // placement rotation, each entry rounded to FP32
  int32_t off;        // shape record offset (doubles) of the daughter
};
static_assert(sizeof(LeafRec) == 128, "LeafRec layout");

// Per placed volume, what a navigation step needs about it and its logical volume in one
// 32-byte load (instead of pv -> lv -> shape -> type/offset and lv -> BVH -> first node).
struct alignas(32) PvRec {
  int32_t lv, shape, type, off; // logical volume, its shape, the shape's type and record offset
  int32_t nd, node0, depth;     // daughters, first BVH node (-1: none), BVH depth (-1: none)
  int32_t child;                // index among the mother's daughters
};
static_assert(sizeof(PvRec) == 32, "PvRec layout");

// Pointers into the device copy of a closed geometry. Passed by value to kernels.
struct DevGeom {
  const double *shape_data; // packed shape records (double-aligned)
  const int32_t *shape_type;
  const int32_t *shape_off;  // record offset (in doubles) per shape id
  const int32_t *lv_shape;
  const int32_t *lv_dstart;  // first entry of the LV's daughters in `daughters`
  const int32_t *lv_nd;
  const int32_t *lv_bvh;     // BVH index of the LV, -1 without daughters
  const int32_t *daughters;  // placed-volume ids in daughter order
  const int32_t *pv_lv;
  const int32_t *pv_child;
  const Xform *pv_xf;
  const int32_t *bvh_node0;  // first node of each BVH in the node arrays
  const int32_t *bvh_prim0;  // first prim slot of each BVH (== lv_dstart of its LV)
  const int32_t *node_nchild;
  const int32_t *node_offset; // absolute prim slot
  const double *node_box;     // 6 doubles per node (lo xyz, hi xyz)
  const int32_t *prim_id;     // daughter index (relative to the LV) per prim slot
  const double *prim_box;     // 6 doubles per daughter slot (indexed lv_dstart + daughter index)
  const NodeF *node_f;        // FP32 node records (bounds rounded outward)
  const float *prim_box_f;    // FP32 daughter boxes (6 floats per slot, rounded outward)
  const float *shape_lbd;     // FP32 bounding descriptor per shape (8 floats, see nav_mixed.cuh)
  const LeafRec *leaf_rec;    // one record per prim slot (absolute slot index)
  const PvRec *pv_rec;        // one record per placed volume
  const uint32_t *nav;        // NavIndex table
  uint32_t nav_words;
  const int32_t *lv_depth;    // BVH depth per LV (-1: no BVH)
  const int32_t *dau_slot3;   // depth-3 subtree (0..7) of each daughter slot's leaf, or -1
  const double *shape_bbox;   // 6 doubles per shape: its bounding box (Extent: lo xyz, hi xyz)
  uint32_t type_mask;         // bit t set: the geometry holds a shape of type t
  int32_t world_pv;
  int32_t max_depth;
  int32_t n_pv;
  int32_t n_lv;
};

} // namespace vg

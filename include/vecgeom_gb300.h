/*
 * vecgeom_gb300 — C ABI of the GB300 (sm_103a) implementation of VecGeom's data-parallel
 * query path: per-track SoA shape queries and the BVH navigation step.
 *
 * Conventions shared by every entry point
 *  - Functions return VG_OK (0) or a negative VG_E* code; vg_last_error() describes the
 *    last failure of the calling thread.
 *  - Query arrays are DEVICE pointers owned by the caller (structure-of-arrays, FP64, like
 *    vecgeom::SOA3D<double>, VecGeom/base/SOA3D.h:36-41). `stream` is a cudaStream_t
 *    (NULL = the legacy default stream); calls are asynchronous with respect to the host.
 *  - Results follow the reference's value conventions: Inside -> 1 inside, 2 surface,
 *    3 outside (EnumInside, VecGeom/base/Global.h:71-79); a miss is 1.7976931348623157e308
 *    (kInfLength); DistanceToOut of an outside point is -1; SafetyToIn is negative inside
 *    and SafetyToOut negative outside.
 *  - Placed-volume and logical-volume ids are assigned in creation order exactly as the
 *    reference does (VPlacedVolume ids: source/PlacedVolume.cpp:32; child ids:
 *    source/LogicalVolume.cpp:142-148), so states are comparable across implementations.
 */
#ifndef VECGEOM_GB300_H
#define VECGEOM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
#define VG_OK 0
#define VG_EINVAL (-1)   /* invalid argument / id / state                   */
#define VG_ECUDA (-2)    /* CUDA runtime error (see vg_last_error)          */
#define VG_ESTATE (-3)   /* geometry not closed, already closed, no world   */
#define VG_ENOMEM (-4)   /* allocation failed                               */

/* Per-track status written by navigation entry points (nullable `status` arrays). */
#define VG_TRACK_OK 0
#define VG_TRACK_ERR_STACK 1 /* BVH traversal stack bound reached */
#define VG_TRACK_ERR_ITER 2  /* locate/relocate loop bound reached */
#define VG_TRACK_ERR_STATE 3 /* input state outside the world       */

/* Shape type tags */
#define VG_SHAPE_BOX 1
#define VG_SHAPE_TUBE 2
#define VG_SHAPE_CONE 3
#define VG_SHAPE_POLYCONE 4
#define VG_SHAPE_POLYHEDRON 5
#define VG_SHAPE_TORUS2 6
#define VG_SHAPE_TRD 7
#define VG_SHAPE_BOOLEAN_SUBTRACTION 8
#define VG_SHAPE_TRAPEZOID 9
#define VG_SHAPE_CUT_TUBE 10
#define VG_SHAPE_SPHERE 11
#define VG_SHAPE_GENTRAP 12
#define VG_SHAPE_HYPE 13

/* Precision flags for queries and navigation */
#define VG_PREC_FP64 0u  /* plain FP64: results identical to the reference's FP64 path          */
#define VG_PREC_MIXED 1u /* FP32 bulk arithmetic with FP64 guard band and FP64 recompute        */

/* Scheduling flags for the navigation step (OR-ed with a precision flag). They change the
 * order in which the device visits tracks, never a track's result (outputs stay at each
 * track's own index). They need a workspace: vg_nav_compute_step_and_next_volume_ws, or
 * the host entry point, which keeps one in the handle. The reference has no counterpart:
 * its SoA navigator loops over tracks in input order (VNavigator.h:128-132). */
#define VG_NAV_SORT 2u  /* radix-sort tracks by (logical volume, Morton cell of the position)   */
#define VG_NAV_QUEUE 4u /* persistent kernel, warps take 32-track chunks from a global counter  */
#define VG_NAV_LEARNED 8u /* explore the BVH subtree proposed by the attached model first       */

/* Navigation state: bit-identical to vecgeom::NavStateIndex {NavIndex_t fNavInd;
 * NavIndex_t fLastExited; bool fOnBoundary;} (VecGeom/navigation/NavStateIndex.h:39-41). */
typedef struct vg_navstate {
  uint32_t nav_ind;
  uint32_t last_exited;
  uint8_t on_boundary;
  uint8_t pad[3];
} vg_navstate;

typedef struct vg_geom vg_geom; /* opaque geometry handle */

const char *vg_last_error(void);
const char *vg_version(void);

/* ---------------------------------------------------------------- geometry construction
 * Replaces the construction half of the reference API: UnplacedBox/UnplacedTube/...
 * constructors, LogicalVolume (VecGeom/volumes/LogicalVolume.h:87-203),
 * LogicalVolume::PlaceDaughter (source/LogicalVolume.cpp:125-155), LogicalVolume::Place,
 * GeoManager::SetWorld + CloseGeometry (source/GeoManager.cpp:192-240) and
 * BVHManager::Init (source/BVHManager.cpp:24-30). Closing builds the daughter boxes, one
 * BVH per logical volume with daughters, the NavIndex table, and uploads the flattened
 * geometry to the current CUDA device (this replaces CudaManager::LoadGeometry/Synchronize,
 * management/CudaManager.h:115-124). A closed geometry is immutable and may be shared by
 * concurrent calls on different streams. */
int vg_geom_create(vg_geom **out);
void vg_geom_destroy(vg_geom *g);

/* Shape constructors; return the shape id (>= 0) or a negative VG_E* code.
 * Units: mm and radians. Parameter meaning follows the reference constructors cited. */
/* UnplacedBox(dx, dy, dz): half-lengths (VecGeom/volumes/BoxStruct.h:19-27) */
int32_t vg_geom_add_box(vg_geom *g, double dx, double dy, double dz);
/* UnplacedTube(rmin, rmax, dz, sphi, dphi) (VecGeom/volumes/UnplacedTube.h:28-34) */
int32_t vg_geom_add_tube(vg_geom *g, double rmin, double rmax, double dz, double sphi, double dphi);
/* UnplacedCone(rmin1, rmax1, rmin2, rmax2, dz, sphi, dphi) (VecGeom/volumes/ConeStruct.h:327-336) */
int32_t vg_geom_add_cone(vg_geom *g, double rmin1, double rmax1, double rmin2, double rmax2, double dz, double sphi,
                         double dphi);
/* UnplacedPolycone(sphi, dphi, nz, z[], rmin[], rmax[]) (VecGeom/volumes/UnplacedPolycone.h) */
int32_t vg_geom_add_polycone(vg_geom *g, double sphi, double dphi, int32_t nz, const double *z, const double *rmin,
                             const double *rmax);
/* UnplacedPolyhedron(phistart, phidelta, nsides, nz, z[], rmin[], rmax[]) (VecGeom/volumes/UnplacedPolyhedron.h) */
int32_t vg_geom_add_polyhedron(vg_geom *g, double phistart, double phidelta, int32_t nsides, int32_t nz,
                               const double *z, const double *rmin, const double *rmax);
/* UnplacedTorus2(rmin, rmax, rtor, sphi, dphi) (VecGeom/volumes/TorusStruct2.h) */
int32_t vg_geom_add_torus2(vg_geom *g, double rmin, double rmax, double rtor, double sphi, double dphi);
/* UnplacedTrd(dx1, dx2, dy1, dy2, dz) (VecGeom/volumes/TrdStruct.h:20-39) */
int32_t vg_geom_add_trd(vg_geom *g, double dx1, double dx2, double dy1, double dy2, double dz);
/* UnplacedTrapezoid(dz, theta, phi, dy1, dx1, dx2, alpha1, dy2, dx3, dx4, alpha2), angles in
 * radians (VecGeom/volumes/UnplacedTrapezoid.h:56-64). The Trd-, box- and parallelepiped-like
 * constructors of UnplacedTrapezoid.h:90-102 are this call with zero angles / equal sides. */
int32_t vg_geom_add_trap(vg_geom *g, double dz, double theta, double phi, double dy1, double dx1, double dx2,
                         double alpha1, double dy2, double dx3, double dx4, double alpha2);
/* UnplacedTrapezoid(TrapCorners) (VecGeom/volumes/UnplacedTrapezoid.h:84-86): corners[24] = eight
 * (x, y, z) in the order (---) (+--) (-+-) (++-) (--+) (+-+) (-++) (+++); dz is the last z. */
int32_t vg_geom_add_trap_corners(vg_geom *g, const double *corners);
/* A trapezoid from its half length and side planes exactly as an existing UnplacedTrapezoid
 * holds them (TrapezoidStruct.h:20-63: fDz and GetPlane(i) for i = 0..3, the planes -Y, +Y,
 * -X, +X): planes[16] = (a, b, c, d) of each plane in that order. Mirrors any trapezoid
 * bit-exactly, whichever constructor made it. */
int32_t vg_geom_add_trap_planes(vg_geom *g, double dz, const double *planes);
/* UnplacedSphere(rmin, rmax, sphi, dphi, stheta, dtheta), angles in radians
 * (VecGeom/volumes/UnplacedSphere.h:40-45, source/UnplacedSphere.cpp:31-37): a spherical
 * shell section; the angles are checked and wrapped as SphereStruct.h:96-170 does. */
int32_t vg_geom_add_sphere(vg_geom *g, double rmin, double rmax, double sphi, double dphi, double stheta,
                           double dtheta);
/* UnplacedHype(rmin, rmax, stIn, stOut, dz) (VecGeom/volumes/UnplacedHype.h:55-61): a tube whose
 * inner and outer surfaces are hyperboloids r^2 = rmin^2 + tan^2(stIn) z^2 and
 * r^2 = rmax^2 + tan^2(stOut) z^2, |z| <= dz; stereo angles in radians. Like the reference,
 * the parameters are not checked. */
int32_t vg_geom_add_hype(vg_geom *g, double rmin, double rmax, double stereo_in, double stereo_out, double dz);
/* UnplacedGenTrap(verticesx[8], verticesy[8], dz) (VecGeom/volumes/UnplacedGenTrap.h:38-45,
 * GenTrapStruct.h Initialize): a generic trapezoid (Arb8) between z = -dz (vertices 0-3)
 * and z = +dz (vertices 4-7), lateral faces planar or twisted. Anticlockwise vertices are
 * reordered clockwise as the reference does; shapes the reference's Initialize reports as
 * errors (opposite orientations, crossing opposite segments, non-convex bases, dz <= 0)
 * are rejected with VG_EINVAL. */
int32_t vg_geom_add_gentrap(vg_geom *g, const double *vertices_x, const double *vertices_y, double dz);
/* UnplacedCutTube(rmin, rmax, dz, sphi, dphi, bx, by, bz, tx, ty, tz)
 * (VecGeom/volumes/UnplacedCutTube.h:54-70): a tube section between two cut planes through
 * (0, 0, -dz) and (0, 0, +dz) with outward normals (bx, by, bz), bz < 0, and (tx, ty, tz),
 * tz > 0 (other normals are rejected with VG_EINVAL, as the reference throws). */
int32_t vg_geom_add_cut_tube(vg_geom *g, double rmin, double rmax, double dz, double sphi, double dphi, double bx,
                             double by, double bz, double tx, double ty, double tz);
/* UnplacedBooleanVolume<kSubtraction>(left, right): operands are placed volumes created
 * with vg_geom_place (VecGeom/volumes/BooleanStruct.h:19-33) */
int32_t vg_geom_add_boolean_subtraction(vg_geom *g, int32_t left_pv, int32_t right_pv);

/* Save / load a geometry description: the builder calls made on `g` (shapes, logical
 * volumes, placements, world), in order, to a binary file; loading replays them on a new,
 * empty handle, which gives the same ids, records and tables as the original (the caller
 * then closes it). No reference counterpart: it replaces the rebuild of a closed VecGeom
 * geometry (GeoManager::CloseGeometry, source/GeoManager.cpp:192) when the mirror is reused. */
int vg_geom_save(const vg_geom *g, const char *path);
int vg_geom_load(vg_geom *g, const char *path);

/* LogicalVolume(shape); returns the logical-volume id. */
int32_t vg_geom_add_logical_volume(vg_geom *g, int32_t shape_id);
/* LogicalVolume::Place(transformation): a placed volume with no mother (world, boolean
 * operands). trans[3], rot[9] as Transformation3D(tx,ty,tz,r0..r8): p_master = R p_local + t
 * with R row-major. Returns the placed-volume id. */
int32_t vg_geom_place(vg_geom *g, int32_t lv, const double trans[3], const double rot[9]);
/* mother_lv.PlaceDaughter(lv, transformation); returns the placed-volume id. */
int32_t vg_geom_place_daughter(vg_geom *g, int32_t mother_lv, int32_t lv, const double trans[3], const double rot[9]);
/* GeoManager::SetWorld */
int vg_geom_set_world(vg_geom *g, int32_t world_pv);
/* Host half of the close: daughter boxes (source/ABBoxManager.cpp:109-140), the BVHs
 * (source/BVH.cpp:48-87) and the NavIndex table (source/NavIndexTable.cpp:9-84), without
 * touching the GPU; the introspection calls below need only this. */
int vg_geom_build(vg_geom *g);
/* GeoManager::CloseGeometry + BVHManager::Init + device upload (builds first if needed) */
int vg_geom_close(vg_geom *g);
/* Introspection of a built geometry (host copies). */
int vg_geom_info(const vg_geom *g, int32_t *n_shapes, int32_t *n_lv, int32_t *n_pv, int32_t *max_depth,
                 size_t *nav_table_words, size_t *device_bytes);
int vg_geom_nav_table(const vg_geom *g, uint32_t *out, size_t words);
int vg_geom_bvh_sizes(const vg_geom *g, int32_t lv, int32_t *n_nodes, int32_t *n_prims, int32_t *depth);
int vg_geom_bvh_arrays(const vg_geom *g, int32_t lv, int32_t *prim_id, int32_t *offset, int32_t *nchild,
                       double *node_box6, double *prim_box6);
int vg_geom_shape_extent(const vg_geom *g, int32_t shape_id, double lo[3], double hi[3]);

/* ---------------------------------------------------------------- SoA shape queries
 * Replace the SoA virtuals of VPlacedVolume (VecGeom/volumes/PlacedVolume.h:271-425):
 *   Inside(SOA3D const&, Inside_t*)                        -> vg_placed_inside        (:299)
 *   Contains(SOA3D const&, bool*)                          -> vg_placed_contains      (:273)
 *   DistanceToIn(SOA3D const&, SOA3D const&, Precision const* step_max, Precision*)
 *                                                          -> vg_placed_distance_to_in  (:332)
 *   DistanceToOut(SOA3D const&, SOA3D const&, step_max*, out*) -> vg_placed_distance_to_out (:372)
 *   SafetyToIn(SOA3D const&, Precision*)                   -> vg_placed_safety_to_in  (:405)
 *   SafetyToOut(SOA3D const&, Precision*)                  -> vg_placed_safety_to_out (:421)
 * Inside, Contains, DistanceToIn and SafetyToIn take points in the mother frame (the placed
 * volume's transformation is applied); DistanceToOut and SafetyToOut take local points, as
 * in the reference (VecGeom/volumes/PlacedVolImplHelper.h:70-123). `step_max` may be NULL
 * (the shapes ignore it, as the reference's do). `flags`: VG_PREC_FP64 or VG_PREC_MIXED. */
int vg_placed_inside(const vg_geom *g, int32_t pv, const double *x, const double *y, const double *z, size_t n,
                     int32_t *out, uint32_t flags, void *stream);
int vg_placed_contains(const vg_geom *g, int32_t pv, const double *x, const double *y, const double *z, size_t n,
                       uint8_t *out, uint32_t flags, void *stream);
int vg_placed_distance_to_in(const vg_geom *g, int32_t pv, const double *x, const double *y, const double *z,
                             const double *dx, const double *dy, const double *dz, const double *step_max, size_t n,
                             double *out, uint32_t flags, void *stream);
int vg_placed_distance_to_out(const vg_geom *g, int32_t pv, const double *x, const double *y, const double *z,
                              const double *dx, const double *dy, const double *dz, const double *step_max, size_t n,
                              double *out, uint32_t flags, void *stream);
int vg_placed_safety_to_in(const vg_geom *g, int32_t pv, const double *x, const double *y, const double *z, size_t n,
                           double *out, uint32_t flags, void *stream);
int vg_placed_safety_to_out(const vg_geom *g, int32_t pv, const double *x, const double *y, const double *z, size_t n,
                            double *out, uint32_t flags, void *stream);

/* ---------------------------------------------------------------- unplaced SoA queries
 * The same six queries on a shape by id, with points and directions in the shape's own frame
 * (no transformation applied), for the VUnplacedVolume interface
 * (VecGeom/volumes/UnplacedVolume.h): Contains (:89), Inside (:96), DistanceToIn (:192),
 * DistanceToOut(SOA3D, SOA3D, step_max*, out*) (:144), SafetyToIn (:223),
 * SafetyToOut(SOA3D, out*) (:179). Arguments and results as for the placed queries. */
int vg_shape_inside(const vg_geom *g, int32_t shape, const double *x, const double *y, const double *z, size_t n,
                    int32_t *out, uint32_t flags, void *stream);
int vg_shape_contains(const vg_geom *g, int32_t shape, const double *x, const double *y, const double *z, size_t n,
                      uint8_t *out, uint32_t flags, void *stream);
int vg_shape_distance_to_in(const vg_geom *g, int32_t shape, const double *x, const double *y, const double *z,
                            const double *dx, const double *dy, const double *dz, const double *step_max, size_t n,
                            double *out, uint32_t flags, void *stream);
int vg_shape_distance_to_out(const vg_geom *g, int32_t shape, const double *x, const double *y, const double *z,
                             const double *dx, const double *dy, const double *dz, const double *step_max, size_t n,
                             double *out, uint32_t flags, void *stream);
int vg_shape_safety_to_in(const vg_geom *g, int32_t shape, const double *x, const double *y, const double *z,
                          size_t n, double *out, uint32_t flags, void *stream);
int vg_shape_safety_to_out(const vg_geom *g, int32_t shape, const double *x, const double *y, const double *z,
                           size_t n, double *out, uint32_t flags, void *stream);

/* ---------------------------------------------------------------- navigation
 * vg_nav_locate_point replaces GlobalLocator::LocateGlobalPoint(world, p, state, true)
 * (VecGeom/navigation/GlobalLocator.h:35-82) with BVHLevelLocator on every logical volume
 * (VecGeom/navigation/BVHLevelLocator.h:44-48). Points outside the world give nav_ind 0. */
int vg_nav_locate_point(const vg_geom *g, const double *x, const double *y, const double *z, size_t n,
                        vg_navstate *out, void *stream);

/* vg_nav_approach_next_daughter replaces BVH::ApproachNextDaughter(localpoint, localdir, step,
 * last) (VecGeom/base/BVH.h:147-159, source/BVH.cpp:394-449), called per track in the frame of
 * its state's volume (the state's global-to-local matrix) with `last` = the state's last-exited
 * volume, as the step passes it to CheckDaughterIntersections. step[] is in/out: on entry the
 * largest distance of interest, on exit lowered to the distance at which the ray first reaches
 * a daughter's bounding box (VUnplacedVolume::ApproachSolid, UnplacedVolume.h:272-280).
 * status[] (nullable) gets VG_TRACK_OK, or an error code with step[] left unchanged.
 * Device pointers; plain FP64, results identical to the reference's FP64 arithmetic. */
int vg_nav_approach_next_daughter(const vg_geom *g, const double *x, const double *y, const double *z,
                                  const double *dx, const double *dy, const double *dz, const vg_navstate *in,
                                  double *step, int32_t *status, size_t n, void *stream);

/* vg_nav_compute_step_and_next_volume replaces the SoA navigator call
 * VNavigator::ComputeStepsAndPropagatedStates(SOA3D const&, SOA3D const&, Precision const*
 * step_limits, NavigationState const* const* in, NavigationState** out, Precision* steps)
 * (VecGeom/navigation/VNavigator.h:128-132) for BVHNavigator<false>, i.e. per track
 * VNavigatorHelper::ComputeStepAndPropagatedState (VNavigator.h:436-492): DistanceToOut of
 * the current volume, BVH daughter intersection, PrepareOutState, relocation after the
 * boundary. The "next volume" is out[i] (its Top()). `step_limit` may be NULL (no physics
 * limit: kInfLength). `status` (nullable) receives VG_TRACK_* per track. `flags`:
 * VG_PREC_FP64 or VG_PREC_MIXED (same out states; steps within 1e-9 mm of FP64). */
int vg_nav_compute_step_and_next_volume(const vg_geom *g, const double *x, const double *y, const double *z,
                                        const double *dx, const double *dy, const double *dz,
                                        const double *step_limit, const vg_navstate *in, vg_navstate *out,
                                        double *step, int32_t *status, size_t n, uint32_t flags, void *stream);

/* vg_nav_compute_step_and_safety replaces VNavigator::ComputeStepAndSafetyAndPropagatedState
 * (VecGeom/navigation/VNavigator.h:1014-1064) with BVHSafetyEstimator
 * (VecGeom/navigation/BVHSafetyEstimator.h:38-46): per track the isotropic safety of the
 * input point in its volume (the mother's SafetyToOut, lowered by BVH::ComputeSafety over
 * the daughters, VecGeom/base/BVH.h:172-209) and the step as above. The safety is FP64 in
 * both precisions; `flags` (VG_PREC_FP64 / VG_PREC_MIXED) selects the step's arithmetic. */
int vg_nav_compute_step_and_safety(const vg_geom *g, const double *x, const double *y, const double *z,
                                   const double *dx, const double *dy, const double *dz, const double *step_limit,
                                   const vg_navstate *in, vg_navstate *out, double *step, double *safety,
                                   int32_t *status, size_t n, uint32_t flags, void *stream);

/* The same step with scheduling flags. `workspace` is device memory of at least
 * vg_nav_step_workspace_bytes(n, flags) bytes (256-byte aligned), used by this call only
 * until the stream reaches its end; concurrent calls need separate workspaces. With
 * flags < VG_NAV_SORT no workspace is needed and the call equals the one above.
 * `nodes_visited` (nullable) receives the BVH nodes the daughter search visited per track
 * (the traversal-cost figure of the learned proposal). */
size_t vg_nav_step_workspace_bytes(size_t n, uint32_t flags);
int vg_nav_compute_step_and_next_volume_ws(const vg_geom *g, const double *x, const double *y, const double *z,
                                           const double *dx, const double *dy, const double *dz,
                                           const double *step_limit, const vg_navstate *in, vg_navstate *out,
                                           double *step, int32_t *status, int32_t *nodes_visited, size_t n,
                                           uint32_t flags, void *workspace, size_t workspace_bytes, void *stream);

/* The scheduled step without any allocation and without a caller workspace: scratch is a
 * fixed 41.5 MiB device array inside the library (capacity 2^20 tracks per call with any
 * flags, VG_NAV_LEARNED's proposal slots included; larger n is rejected with VG_EINVAL).
 * No reference counterpart: it exists for callers that may not allocate device memory on
 * the step path. Calls that overlap in time share the scratch and race, so callers
 * serialise them; the first call on a device looks the scratch up and belongs in setup,
 * before any stream capture. The looked-up address is kept for the life of the process:
 * after cudaDeviceReset (or a reset of the primary context) it is stale, so a process
 * that resets a device must not call this entry point on it again. Same flags and results
 * as vg_nav_compute_step_and_next_volume_ws. */
int vg_nav_compute_step_and_next_volume_noalloc(const vg_geom *g, const double *x, const double *y, const double *z,
                                                const double *dx, const double *dy, const double *dz,
                                                const double *step_limit, const vg_navstate *in, vg_navstate *out,
                                                double *step, int32_t *status, size_t n, uint32_t flags,
                                                void *stream);

/* Transport stream (config-5 style): every track steps until it leaves the world or has made
 * max_steps steps, as the reference's navigator would be driven by a straight-line
 * transport loop (per step VNavigator::ComputeStepAndPropagatedState with no physics limit,
 * then p += step * d). x/y/z and `states` are updated in place; nsteps[i] receives the
 * steps of track i, status[i] a VG_TRACK_* give-up code (0 normally). Tracks below
 * trace_tracks record each step's out-state and length at [i * max_steps + k] of
 * trace_states / trace_steps. Each iteration steps all live tracks with one persistent
 * kernel (refilled from a compacted list of survivors), after sorting them (VG_NAV_SORT)
 * and computing proposals (VG_NAV_LEARNED) if asked. The iterations run in a device-side
 * loop (a CUDA graph whose while-node repeats them until the stream ends; the live count
 * never returns to the host in between). With VG_NAV_QUEUE, once fewer tracks are alive
 * than 512 per SM, the rest runs as one pass in which every thread steps a track to its
 * end and then takes the next (same results, no per-iteration sort). *iterations
 * (nullable) receives the number of passes (iterations, plus one for such a tail pass).
 * Synchronises the stream; builds and frees its graph on every call. No single reference
 * counterpart. */
size_t vg_nav_transport_workspace_bytes(size_t n, uint32_t flags);
int vg_nav_transport(const vg_geom *g, double *x, double *y, double *z, const double *dx, const double *dy,
                     const double *dz, vg_navstate *states, size_t n, int32_t max_steps, uint32_t flags,
                     int32_t *nsteps, int32_t *status, vg_navstate *trace_states, double *trace_steps,
                     size_t trace_tracks, int32_t *iterations, void *workspace, size_t workspace_bytes, void *stream);

/* The visiting order VG_NAV_SORT uses, for callers that want to reorder their own track
 * arrays: key = logical-volume id of the state's top volume << 3*cell_bits | Morton code of
 * the position's cell (cell_bits per axis over the world box; cell = (float)(c - lo) * scale
 * truncated and clamped to [0, 2^cell_bits - 1]); states outside the world get 0xffffffff.
 * `order` receives the track indices sorted stably by key, `keys` (nullable) the sorted
 * keys. The workspace is sized by vg_nav_step_workspace_bytes(n, VG_NAV_SORT). No
 * reference counterpart. */
int vg_nav_sort_tracks(const vg_geom *g, const double *x, const double *y, const double *z, const vg_navstate *in,
                       size_t n, uint32_t *order, uint32_t *keys, void *workspace, size_t workspace_bytes,
                       void *stream);
int vg_nav_sort_key_params(const vg_geom *g, float lo[3], float scale[3], int32_t *cell_bits, int32_t *lv_bits);
/* Tuning knobs of the scheduled step (results never depend on them): `cell_bits`, the
 * Morton bits per axis of the sort key (1..10; 0 = default, the most that fit beside the
 * logical-volume id; fewer bits mean fewer radix passes and coarser cells), and
 * `queue_blocks_per_sm`, the configuration of the VG_NAV_QUEUE kernel (1: blocks of 256
 * threads, one per SM, full register budget; 2: two per SM, half the registers, twice the
 * resident warps; 3: blocks of 128 threads, three per SM, 168 registers; 4: blocks of 128
 * threads, five per SM, 20 resident warps at 102 registers; 5-8: the budgets of 1-4 with the
 * step split into two kernels, the step up to the boundary and then the relocation, over
 * the same visiting order; 0 = 1). Set before sorted calls are in flight. */
int vg_nav_set_tuning(vg_geom *g, int32_t cell_bits, int32_t queue_blocks_per_sm);

/* ---------------------------------------------------------------- learned proposal
 * No reference counterpart. A small MLP (80 -> 64 -> 64 -> 16, ReLU, BF16 weights for
 * inference) predicts for a track in a logical volume whose BVH has depth >= 3 which of
 * the 8 depth-3 BVH subtrees holds the first daughter the ray hits (or none). With
 * VG_NAV_LEARNED the step explores the proposed subtree first, which tightens the step
 * bound early; the full traversal still decides, so results do not depend on the model.
 * vg_learn_features writes 80 FP32 features per track (`feat`, n x 80), the logical volume
 * (`lv`, -1 where no proposal applies) and, if `label` is given, the training label from
 * the plain FP64 traversal (0..7 subtree, 8 none, -1 not applicable). Training consumes
 * only samples with lv >= 0 and 0 <= label <= 8: callers pass that subset. Gradients and
 * parameters use one flat FP32 layout: W1[64][80], b1[64], W2[64][64], b2[64], W3[16][64],
 * b3[16], E[n_lv][16]. All arrays are device memory unless stated. */
typedef struct vg_mlp vg_mlp;
int vg_mlp_create(const vg_geom *g, uint64_t seed, vg_mlp **out);
void vg_mlp_destroy(vg_mlp *m);
size_t vg_mlp_param_count(const vg_mlp *m);
int vg_mlp_get_params(const vg_mlp *m, float *host, size_t n); /* host buffer */
int vg_mlp_set_params(vg_mlp *m, const float *host, size_t n); /* host buffer; resets Adam */
int vg_learn_features(const vg_geom *g, const double *x, const double *y, const double *z, const double *dx,
                      const double *dy, const double *dz, const vg_navstate *in, size_t n, float *feat, int32_t *lv,
                      int8_t *label, void *stream);
/* Forward + backward over all n samples: mean softmax cross-entropy gradients (flat
 * layout) and the summed loss. Synchronises the stream. */
int vg_mlp_gradients(vg_mlp *m, const float *feat, const int32_t *lv, const int8_t *label, size_t n, float *grads,
                     float *loss, void *stream);
/* Adam (0.9, 0.999, 1e-8) over shuffled mini-batches; epoch_loss (host, nullable) gets the
 * mean loss of each epoch. Refreshes the BF16 inference copy. Synchronises the stream. */
int vg_mlp_train(vg_mlp *m, const float *feat, const int32_t *lv, const int8_t *label, size_t n, int32_t epochs,
                 int32_t batch, float lr, uint64_t seed, float *epoch_loss, void *stream);
/* Proposals from features: slot 0..7, or -1 for "none" / no proposal; logits (nullable,
 * n x 16 FP32). flags 0: SIMT kernel; 1: tensor-core kernel (tcgen05, same semantics). */
int vg_mlp_infer(const vg_mlp *m, const float *feat, const int32_t *lv, size_t n, int8_t *slot, float *logits,
                 uint32_t flags, void *stream);
/* Model used by steps with VG_NAV_LEARNED (NULL detaches). The model must outlive its use. */
int vg_geom_set_proposer(vg_geom *g, const vg_mlp *m);
/* Kernel VG_NAV_LEARNED uses for its proposals: 1 tensor-core (default), 0 SIMT. */
int vg_nav_set_proposal_kernel(vg_geom *g, int32_t tensor);
/* Reads and clears the model's error flag: 1 if a tensor-core kernel's bounded wait for its
 * MMA gave up (its proposals are then incomplete; step results are unaffected). */
int vg_mlp_error(const vg_mlp *m, int32_t *error);
/* The proposals VG_NAV_LEARNED computes inside the step (features + attached model), for
 * n tracks: slot 0..7 or -1. flags 0: SIMT kernel; 1: tensor-core kernel. */
int vg_nav_propose(const vg_geom *g, const double *x, const double *y, const double *z, const double *dx,
                   const double *dy, const double *dz, const vg_navstate *in, size_t n, int8_t *slot, uint32_t flags,
                   void *stream);

/* Same step with HOST arrays, the form the reference's own SoA navigator interface takes
 * (VNavigator::ComputeStepsAndPropagatedStates, VNavigator.h:128-132): inputs are copied to
 * device staging buffers owned by the handle (allocated on first use, grown on demand,
 * serialised by a lock), the kernel runs on `stream`, results are copied back and the call
 * returns after the stream has synchronised. Pinned host memory gives full copy bandwidth.
 * `flags` may include VG_NAV_SORT / VG_NAV_QUEUE (the workspace is part of the staging). */
int vg_nav_compute_step_and_next_volume_host(vg_geom *g, const double *x, const double *y, const double *z,
                                             const double *dx, const double *dy, const double *dz,
                                             const double *step_limit, const vg_navstate *in, vg_navstate *out,
                                             double *step, int32_t *status, size_t n, uint32_t flags, void *stream);

/* ---------------------------------------------------------------- measurement utility
 * FP64 FMA issue rate of the current device (DFMA instructions per second), timed on
 * `stream` with CUDA events: the peak against which the navigation kernels' FP64 roofline
 * is stated. No reference counterpart (a measurement aid, not part of the query path). */
int vg_device_fp64_rate(double *fma_per_s, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* VECGEOM_GB300_H */

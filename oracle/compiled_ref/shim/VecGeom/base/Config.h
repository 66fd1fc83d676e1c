// ORACLE — TEST INFRASTRUCTURE ONLY. The configuration header the reference's CMake would
// generate from VecGeom/base/Config.h.in, written for the compiled-reference oracle with
// the settings the device path reproduces: scalar backend, double precision, volume
// specialisation off, PlaneShell on, transformations in place, indexed navigation states
// with the navigation index table on, no CUDA, ROOT, Geant4, Embree or GDML.
#ifndef VECGEOM_BASE_CONFIG_H_
#define VECGEOM_BASE_CONFIG_H_

#define VECGEOM_SCALAR
#define VECGEOM_CUDA_NO_VOLUME_SPECIALIZATION
#define VECGEOM_NO_SPECIALIZATION
#define VECGEOM_INPLACE_TRANSFORMATIONS
#define VECGEOM_PLANESHELL
#define VECGEOM_USE_INDEXEDNAVSTATES
#define VECGEOM_USE_NAVINDEX

#endif

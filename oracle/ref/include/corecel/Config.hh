// Hand-written configuration header for compiling the reference's host
// stepping loop as a CPU oracle. It stands in for the file that the
// reference's CMake configure step writes from src/corecel/Config.hh.in:23-62,
// using the option numbering of cmake/CeleritasUtils.cmake:631-659
// (disabled options 0, available options counted from 1).
//
// Configuration: FP64 reals, CGS units, ORANGE geometry, XORWOW RNG, no
// OpenMP, host only (no CUDA/HIP), no optional external libraries.
#pragma once

#define CELERITAS_USE_CUDA 0
#define CELERITAS_USE_GEANT4 0
#define CELERITAS_USE_HEPMC3 0
#define CELERITAS_USE_HIP 0
#define CELERITAS_USE_MPI 0
#define CELERITAS_USE_OPENMP 0
#define CELERITAS_USE_PERFETTO 0
#define CELERITAS_USE_PNG 0
#define CELERITAS_USE_ROOT 0
#define CELERITAS_USE_VECGEOM 0

#define CELERITAS_DEBUG 0
#define CELERITAS_DEVICE_DEBUG 0

#ifndef CELERITAS_ORACLE_REAL_FLOAT
#    define CELERITAS_REAL_TYPE_DOUBLE 1
#    define CELERITAS_REAL_TYPE_FLOAT 2
#else
#    define CELERITAS_REAL_TYPE_DOUBLE 1
#    define CELERITAS_REAL_TYPE_FLOAT 2
#endif
#ifdef CELERITAS_ORACLE_REAL_FLOAT
#    define CELERITAS_REAL_TYPE CELERITAS_REAL_TYPE_FLOAT
#else
#    define CELERITAS_REAL_TYPE CELERITAS_REAL_TYPE_DOUBLE
#endif

#define CELERITAS_UNITS_CGS 1
#define CELERITAS_UNITS_SI 2
#define CELERITAS_UNITS_CLHEP 3
#define CELERITAS_UNITS CELERITAS_UNITS_CGS

#define CELERITAS_OPENMP_EVENT 0
#define CELERITAS_OPENMP_TRACK 0
#define CELERITAS_OPENMP_DISABLED 1
#define CELERITAS_OPENMP CELERITAS_OPENMP_DISABLED

#define CELERITAS_CORE_GEO_VECGEOM 0
#define CELERITAS_CORE_GEO_GEANT4 0
#define CELERITAS_CORE_GEO_ORANGE 1
#define CELERITAS_CORE_GEO CELERITAS_CORE_GEO_ORANGE

#define CELERITAS_CORE_RNG_CURAND 0
#define CELERITAS_CORE_RNG_HIPRAND 0
#define CELERITAS_CORE_RNG_XORWOW 1
#define CELERITAS_CORE_RNG CELERITAS_CORE_RNG_XORWOW

#define CELERITAS_MAX_BLOCK_SIZE 0

inline constexpr char celeritas_build_type[] = "Release";
inline constexpr char celeritas_hostname[] = "oracle";
#ifdef CELERITAS_ORACLE_REAL_FLOAT
inline constexpr char celeritas_real_type[] = "float";
#else
inline constexpr char celeritas_real_type[] = "double";
#endif
inline constexpr char celeritas_units[] = "CGS";
inline constexpr char celeritas_openmp[] = "disabled";
inline constexpr char celeritas_core_geo[] = "ORANGE";
inline constexpr char celeritas_core_rng[] = "xorwow";
inline constexpr char celeritas_clhep_version[] = "";
inline constexpr char celeritas_geant4_version[] = "";
inline constexpr char celeritas_vecgeom_version[] = "";

#define CELERITAS_HAVE_ROCTX 0

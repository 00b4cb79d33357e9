// Hand-written version header for the CPU-oracle build of the reference; it
// stands in for the file generated from src/corecel/Version.hh.in (release
// series 0.5).
#pragma once

#define CELERITAS_VERSION 0x000500

inline constexpr char celeritas_version[] = "0.5.0";
inline constexpr int celeritas_version_major = 0;
inline constexpr int celeritas_version_minor = 5;
inline constexpr int celeritas_version_patch = 0;

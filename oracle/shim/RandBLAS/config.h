// Configuration header for compiling the RandBLAS headers without CMake, written the way
// the reference's RandBLAS/config.h.in instructs ("copy this file to config.h and
// substitute"): OpenMP on, MKL off (test infrastructure).
#pragma once
#define RandBLAS_HAS_OpenMP
#define RandBLAS_FULL_VERSION "1.1.0-shim"
#define RandBLAS_VERSION_MAJOR 1
#define RandBLAS_VERSION_MINOR 1
#define RandBLAS_VERSION_PATCH 0

/*
 * p3dfft3config.h -- configuration header for building the reference library here
 * (oracle/_ref), in place of the one its configure script would generate from
 * p3dfft3config.h.in.  TEST INFRASTRUCTURE ONLY.
 *
 * FFTW back end with the ESTIMATE planner flag (the shim plans nothing, so the flag only keys
 * the reference's plan cache, build/templ.C:1243-1246); GNU compiler; no timers.
 */
#ifndef ORC_P3DFFT3CONFIG_H
#define ORC_P3DFFT3CONFIG_H
#define FFTW 1
#define FFTW_FLAG_ESTIMATE 1
#define GNU 1
#define HAVE_STDLIB_H 1
#define HAVE_STRING_H 1
#define PACKAGE "p3dfft++"
#define VERSION "3 (reference, built against the oracle's FFTW-API shim)"
#endif

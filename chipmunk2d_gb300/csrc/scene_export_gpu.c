/*
 * scene_export_gpu.c -- the state-export names the tests and the benchmark
 * call on every implementation of the API (cpx_dump_bodies, ...), mapped
 * onto the GPU library's cpGpuDebug* entry points.  Built into the
 * test-side workload library (libcpx_scenes.so) with scenes.c, not into
 * the product.
 */
#include "../../include/chipmunk_gb300.h"

int cpx_dump_bodies(cpSpace *sp, double *out, int max) { return cpGpuDebugBodies(sp, out, max); }
int cpx_dump_arbiters(cpSpace *sp, double *out, int max) { return cpGpuDebugArbiters(sp, out, max); }
int cpx_dump_constraints(cpSpace *sp, double *out, int max) { return cpGpuDebugConstraints(sp, out, max); }
int cpx_set_bodies(cpSpace *sp, const double *in, int count) { return cpGpuDebugSetBodies(sp, in, count); }
int cpx_dump_candidates(cpSpace *sp, int *out, int max) { return cpGpuDebugCandidates(sp, out, max); }

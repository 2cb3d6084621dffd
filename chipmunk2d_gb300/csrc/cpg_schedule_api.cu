/*
 * cpg_schedule_api.cu -- standalone exact-order sweep scheduler.
 *
 * A sequential-impulse sweep applies its units (contacts, joints) one after
 * the other (src/cpSpaceStep.c:418-427).  Two units that share no dynamic
 * body commute exactly, so the sweep can run level by level: a unit's level
 * is 1 + the level of the latest earlier unit touching any of its bodies.
 * Every body then sees its updates in the original order and the parallel
 * sweep reproduces the serial one bit for bit.  cpGpuSolveSchedule computes
 * that schedule for any unit sequence given as two body indices per unit
 * (negative = no dynamic body), entirely on the device.
 *
 * Scratch: the per-body "last level" array and the per-unit levels.
 */
#include <cstdio>
#include <cuda_runtime.h>
#include "../../include/chipmunk_gb300.h"

/* Level of every unit; one thread walks the sequence (the recurrence is a
 * scan in unit order).  Then the block counting-sorts units by level. */
__device__ void schedule_levels(const int *bodyA, const int *bodyB, int nunits, int nbodies,
                                int *last, int *level, int *levelStart, int *order, int *nlevels)
{
	for(int b = threadIdx.x; b < nbodies; b += blockDim.x) last[b] = 0;
	__syncthreads();
	if(threadIdx.x == 0){
		int maxl = 0;
		for(int u = 0; u < nunits; u++){
			int a = bodyA[u], b = bodyB[u];
			if(a >= nbodies) a = -1;
			if(b >= nbodies) b = -1;
			int l = 0;
			if(a >= 0 && last[a] > l) l = last[a];
			if(b >= 0 && last[b] > l) l = last[b];
			level[u] = l;
			if(a >= 0) last[a] = l + 1;
			if(b >= 0) last[b] = l + 1;
			if(l + 1 > maxl) maxl = l + 1;
		}
		for(int l = 0; l <= maxl; l++) levelStart[l] = 0;
		for(int u = 0; u < nunits; u++) levelStart[level[u] + 1]++;
		for(int l = 0; l < maxl; l++) levelStart[l + 1] += levelStart[l];
		/* stable scatter with levelStart as the cursors, shifted back after */
		for(int u = 0; u < nunits; u++){
			int l = level[u];
			order[levelStart[l]] = u;
			levelStart[l]++;
		}
		for(int l = maxl; l > 0; l--) levelStart[l] = levelStart[l - 1];
		levelStart[0] = 0;
		*nlevels = maxl;
	}
	__syncthreads();
}

__global__ void k_schedule_api(const int *bodyA, const int *bodyB, int nunits, int nbodies,
                               int *last, int *level, int *levelStart, int *order, int *nlevels)
{
	schedule_levels(bodyA, bodyB, nunits, nbodies, last, level, levelStart, order, nlevels);
}

/* levelStart always receives levelStart[0] = 0, even for an empty
 * sequence, so it must be a device array of nunits + 1 ints whatever
 * nunits is; order and the body arrays are only touched when nunits > 0. */
static bool schedule_args_ok(const int *bodyA, const int *bodyB, int nunits, int nbodies,
                             const int *levelStart, const int *order, const int *nlevels)
{
	if(nunits < 0 || nbodies < 0 || !levelStart || !nlevels) return false;
	if(nunits > 0 && (!bodyA || !bodyB || !order)) return false;
	return true;
}

extern "C" int cpGpuSolveSchedule(const int *bodyA, const int *bodyB, int nunits, int nbodies,
                                  int *levelStart, int *order, int *nlevels, void *stream)
{
	if(!schedule_args_ok(bodyA, bodyB, nunits, nbodies, levelStart, order, nlevels)) return CP_GPU_ERR_ARGUMENT;
	cudaStream_t st = (cudaStream_t)stream;
	int *scratch = NULL;
	size_t words = (size_t)nbodies + (size_t)nunits + 1;
	if(cudaMallocAsync((void **)&scratch, words*sizeof(int), st) != cudaSuccess) return CP_GPU_ERR_CUDA;
	k_schedule_api<<<1, 256, 0, st>>>(bodyA, bodyB, nunits, nbodies, scratch, scratch + nbodies, levelStart, order, nlevels);
	cudaError_t e = cudaGetLastError();
	cudaFreeAsync(scratch, st);
	return e == cudaSuccess ? CP_GPU_OK : CP_GPU_ERR_CUDA;
}

/* ------------------------------------------------------------------ */
/* Allocation-free variant.
 *
 * Some callers cannot allocate device memory when they need a schedule: a
 * frame loop with a hard time budget (cudaMalloc and cudaMallocAsync may
 * synchronise or take unbounded time), or a host application that owns
 * every device allocation through its own memory manager and forbids
 * libraries from allocating after start-up.  cpGpuSolveScheduleNoAlloc
 * serves them: it runs the same kernel with its scratch in a fixed device
 * array that is part of the library image, so the call itself allocates
 * nothing.  The array (8 MiB) exists on every GPU that loads the library
 * until the process exits.  Calls share it, so calls that overlap on the
 * GPU (different streams, or different host threads) race; the kernel
 * clears the part that must start at zero on every call.
 */
#define CPG_SCHEDULE_STATIC_MAX_BODIES (1 << 20)
#define CPG_SCHEDULE_STATIC_MAX_UNITS (1 << 20)

static __device__ __align__(256) int g_schedule_scratch[CPG_SCHEDULE_STATIC_MAX_BODIES + CPG_SCHEDULE_STATIC_MAX_UNITS];

#define CPG_SCHEDULE_MAX_DEVICES 64
/* Device address of g_schedule_scratch per device; host code cannot use the
 * symbol's name as a device pointer. */
static int *g_schedule_scratch_addr[CPG_SCHEDULE_MAX_DEVICES];

extern "C" int cpGpuSolveScheduleNoAlloc(const int *bodyA, const int *bodyB, int nunits, int nbodies,
                                         int *levelStart, int *order, int *nlevels, void *stream)
{
	if(!schedule_args_ok(bodyA, bodyB, nunits, nbodies, levelStart, order, nlevels)) return CP_GPU_ERR_ARGUMENT;
	if(nunits > CPG_SCHEDULE_STATIC_MAX_UNITS || nbodies > CPG_SCHEDULE_STATIC_MAX_BODIES){
		fprintf(stderr, "cpGpuSolveScheduleNoAlloc: %d units / %d bodies exceed the fixed scratch (%d units, %d bodies)\n",
			nunits, nbodies, CPG_SCHEDULE_STATIC_MAX_UNITS, CPG_SCHEDULE_STATIC_MAX_BODIES);
		return CP_GPU_ERR_ARGUMENT;
	}
	int dev = 0;
	if(cudaGetDevice(&dev) != cudaSuccess) return CP_GPU_ERR_CUDA;
	if(dev < 0 || dev >= CPG_SCHEDULE_MAX_DEVICES) return CP_GPU_ERR_ARGUMENT;
	if(!g_schedule_scratch_addr[dev]){
		/* once per device, with that device current */
		int *ptr = NULL;
		if(cudaGetSymbolAddress((void **)&ptr, g_schedule_scratch) != cudaSuccess || ptr == NULL) return CP_GPU_ERR_CUDA;
		g_schedule_scratch_addr[dev] = ptr;
	}
	int *scratch = g_schedule_scratch_addr[dev];
	cudaStream_t st = (cudaStream_t)stream;
	k_schedule_api<<<1, 256, 0, st>>>(bodyA, bodyB, nunits, nbodies, scratch, scratch + nbodies, levelStart, order, nlevels);
	return cudaGetLastError() == cudaSuccess ? CP_GPU_OK : CP_GPU_ERR_CUDA;
}

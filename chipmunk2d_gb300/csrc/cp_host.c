/*
 * cp_host.c -- host side of libchipmunk_gb300: the Chipmunk2D C API
 * (include/chipmunk_gb300.h) over device-resident simulation state.
 *
 * Objects (bodies, shapes, constraints, spaces) are host structs holding
 * their creation-time data.  The first cpSpaceStep packs the space into a
 * device set (cpg_device.h) and from then on the dynamic state lives in
 * HBM: cpSpaceStep enqueues the step's kernels (cpg_kernels.cu) on the
 * library's stream and returns; getters synchronise and copy state back
 * lazily, setters mark it dirty for upload before the next step.  The
 * index insertions made by cpSpaceAddShape are recorded with the shape's
 * box and body velocity at the time of the call and replayed on the device
 * in the same order, so the device AABB tree grows exactly as the
 * reference's does.
 *
 * There is no CPU fallback: a space that needs a feature the device step
 * does not implement (custom integration callbacks, sleeping) is not
 * stepped and cpGpuGetLastError() reports CP_GPU_ERR_UNSUPPORTED.
 *
 * Host floating-point code (moments, hulls, add-time shape caches, the
 * per-step pow() terms) follows the reference's expressions and is built
 * with -ffp-contract=off so it rounds identically.
 */
#define _GNU_SOURCE
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdarg.h>
#include <cuda_runtime.h>
#include "../../include/chipmunk_gb300.h"
#include "cpg_device.h"

#define INF_ ((cpFloat)INFINITY)

/* ====================================================================
 * Errors
 * ==================================================================== */
const char *cpVersionString = "7.0.3";

static int g_error = CP_GPU_OK;
static char g_errmsg[256] = "";

static void set_error(int code, const char *fmt, ...)
{
	if(g_error == CP_GPU_OK){
		g_error = code;
		va_list ap;
		va_start(ap, fmt);
		vsnprintf(g_errmsg, sizeof(g_errmsg), fmt, ap);
		va_end(ap);
	}
}

int cpGpuGetLastError(void) { int e = g_error; g_error = CP_GPU_OK; return e; }
const char *cpGpuGetLastErrorString(void) { return g_errmsg; }

/* chipmunk.c:31-54 */
void cpMessage(const char *condition, const char *file, int line, int isError, int isHardError, const char *message, ...)
{
	fprintf(stderr, (isError ? "Aborting due to Chipmunk error: " : "Chipmunk warning: "));
	va_list vargs;
	va_start(vargs, message);
	vfprintf(stderr, message, vargs);
	va_end(vargs);
	fprintf(stderr, "\n\tFailed condition: %s\n\tSource:%s:%d\n", condition, file, line);
	(void)isHardError;
}

/* cpAssertHard semantics (chipmunk.h:58): report and abort. */
#define ASSERT_HARD(cond, msg) do { if(!(cond)){ cpMessage(#cond, __FILE__, __LINE__, 1, 1, msg); abort(); } } while(0)

static int cuda_ok(cudaError_t e, const char *what)
{
	if(e == cudaSuccess) return 1;
	set_error(CP_GPU_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
	return 0;
}

/* ====================================================================
 * Scalar helpers (chipmunk_types.h:137-168)
 * ==================================================================== */
static inline cpFloat hmax(cpFloat a, cpFloat b) { return (a > b) ? a : b; }
static inline cpFloat hmin(cpFloat a, cpFloat b) { return (a < b) ? a : b; }
static inline cpFloat habs(cpFloat f) { return (f < 0) ? -f : f; }
static inline cpTransform rigid_inverse(cpTransform t)
{
	return cpTransformNewTranspose(t.d, -t.c, (t.c*t.ty - t.tx*t.d), -t.b, t.a, (t.tx*t.b - t.a*t.ty));
}

/* ====================================================================
 * Objects
 * ==================================================================== */
typedef struct DevSet DevSet;

struct cpBody {
	cpBodyVelocityFunc velocity_func;
	cpBodyPositionFunc position_func;
	cpFloat m, m_inv, i, i_inv;
	cpVect cog, p, v, f;
	cpFloat a, w, t;
	cpTransform transform;
	cpVect v_bias;
	cpFloat w_bias;
	cpFloat idleTime;
	cpDataPointer userData;
	cpSpace *space;
	int index;                 /* world-local device index */
	DevSet *devOwner;          /* the device set `index` refers to */
	unsigned long long pullGen; /* download whose state this struct holds */
	cpShape *shapeList;
	cpConstraint *constraintList;
	/* sleeping (chipmunk_structs.h:90-94): the component root and next
	 * body; the head of the body's list in the contact graph, as an index
	 * of the space's graph pool + 1 (0 = none) */
	cpBody *sleepRoot, *sleepNext;
	int arbList;
};

struct cpShape {
	int kind;
	cpSpace *space;
	cpBody *body;
	cpFloat mass_m, mass_i, mass_area;
	cpVect mass_cog;
	cpBB bb;
	cpBool sensor;
	cpFloat e, u;
	cpVect surfaceV;
	cpDataPointer userData;
	cpCollisionType ctype;
	cpShapeFilter filter;
	cpShape *next, *prev;
	cpHashValue hashid;
	cpFloat r;
	cpVect c, tc;                          /* circle */
	cpVect sa, sb, sn, ta, tb, tn;         /* segment */
	cpVect a_tangent, b_tangent;
	int count;                             /* polygon */
	cpVect *lv, *ln, *gv, *gn;             /* local/world planes */
};

struct cpConstraint {
	int kind;
	cpSpace *space;
	cpBody *a, *b;
	cpConstraint *next_a, *next_b;
	cpFloat maxForce, errorBias, maxBias;
	cpBool collideBodies;
	cpConstraintPreSolveFunc preSolve;
	cpConstraintPostSolveFunc postSolve;
	cpDataPointer userData;
	cpVect anchorA, anchorB;
	cpFloat dist, min, max;
	/* groove, springs, rotary joints (the ratchet's angle, a state the
	 * step updates, lives in rec) */
	cpVect grv_a, grv_b, grv_n;
	cpFloat restLength, restAngle, stiffness, damping;
	cpFloat phase, ratchet, ratio, ratio_inv, rate;
	cpDampedSpringForceFunc springForceFunc;
	cpDampedRotarySpringTorqueFunc springTorqueFunc;
	int index;
	cpgJoint rec;                          /* last downloaded device record */
};

/* Snapshot of a device arbiter, valid until the next step. */
struct cpArbiter {
	cpShape *a, *b;
	cpBody *body_a, *body_b;
	int count, state;
	cpVect n, surface_vr;
	cpFloat e, u;
	cpBool swapped;
	cpgContact c[2];
	/* contact-graph entries only: the device table key, body_a's and
	 * body_b's list links (graph index + 1, 0 = none) and the position in
	 * the arbiter list (-1: not on it) */
	unsigned long long key;
	int prevA, nextA, prevB, nextB;
	int listPos;
	/* collision handlers (chipmunk_structs.h:210-214): those of the last
	 * update, the user data, the device slot of the record */
	cpCollisionHandler *handler, *handlerA, *handlerB;
	cpDataPointer data;
	int slot;
};

struct cpSpace {
	int iterations;
	cpVect gravity;
	cpFloat damping, idleSpeedThreshold, sleepTimeThreshold;
	cpFloat collisionSlop, collisionBias;
	cpTimestamp collisionPersistence;
	cpDataPointer userData;
	cpTimestamp stamp;
	cpFloat curr_dt;
	cpHashValue shapeIDCounter;
	int mode;

	cpBody **dyn; int ndyn, capdyn;
	cpBody **stat; int nstat, capstat;
	/* shapes by hash id: a removed shape leaves its slot NULL, so the
	 * device index of a shape (its hash id) never changes */
	cpShape **shapes; int nshapes, capshapes;
	int nlive;                              /* shapes in the space */
	cpConstraint **cons; int ncons, capcons;
	cpgOp *ops; int nops, capops;           /* insertions not yet on the device */
	cpBody staticBody;

	DevSet *dev;                            /* device set holding this space */
	int world;                              /* index in the set */
	int ownsDev;
	int builtBodies, builtShapes, builtCons;
	int hostStale;                          /* device bodies newer than host */
	int consStale;                          /* device joint records newer than host */
	int shapesStale;                        /* device shape boxes newer than host */
	int bodyDirty, shapeDirty, consDirty;   /* host newer than device */
	int structDirty;                        /* objects added or removed since the device set was built:
	                                           the host holds the state until the next step rebuilds it */
	double jointDt;                         /* dt the joint bias terms were made for */
	unsigned long long editGen;             /* counts object edits through the setters */
	unsigned long hastyThreads;             /* cpHastySpaceSetThreads */
	struct PostStep *post; int npost, cappost, postRunning;   /* cpSpaceAddPostStepCallback */

	cpArbiter *snap; int nsnap, capsnap; int snapValid;
	float phaseMs[8];

	/* sleeping (cpSpaceComponent.c): bodies asleep, in device order after
	 * the dynamic array; the sleeping components' roots; bodies woken while
	 * the space was locked */
	cpBody **slp; int nslp, capslp;
	cpBody **sleeping; int nsleeping, capsleeping;
	cpBody **roused; int nroused, caproused;
	int locked;
	/* the contact graph, kept while sleeping is on: a pool of arbiter
	 * records with their list links, and the arbiter list (pool indices) */
	int graphOn, graphFresh;
	cpArbiter *garb; int ngarb, capgarb;
	int *gfree; int ngfree, capgfree;
	int *glist; int nglist, capglist;
	/* cache edits for the device (key, 1 = out of the cache, stamp) */
	unsigned long long *sedKey; int *sedOp; unsigned *sedStamp; int nsed, capsed;
	int sleepMutated;
	double prevDt;

	/* collision handlers (cpSpace.c:62-103, 378-413): once any is added,
	 * the step runs the callbacks on the host between its device halves */
	cpCollisionHandler defaultHandler;
	int usesWildcards, handlersOn, defaultTouched;
	cpCollisionHandler **handlers; int nhandlers, caphandlers;
	cpArbiter *harb; int capharb;            /* the arbiters of one round of callbacks */
	/* cpSpaceUseSpatialHash: both indices are spatial hashes */
	int useHash, hashCells;
	cpFloat hashDim;
	unsigned long long *udKey; cpDataPointer *udVal; int udCap, udUsed;   /* arbiter user data by key */
};

static void run_post_step_(cpSpace *sp);
static void space_unlock_(cpSpace *sp);
static cpShape *slot_shape_(cpSpace *sp, int slot);

static void push_(void ***arr, int *n, int *cap, void *p)
{
	if(*n == *cap){
		*cap = *cap ? 2*(*cap) : 64;
		*arr = (void **)realloc(*arr, sizeof(void *)*(size_t)(*cap));
	}
	(*arr)[(*n)++] = p;
}

/* ====================================================================
 * Device sets
 * ==================================================================== */
#define CPG_STATS_INTERVAL 16
/* The step parameters are uploaded from pinned memory by an asynchronous
 * copy, so the host must not rewrite a block until that copy has run: the
 * blocks rotate through a ring and each is reused only after its event. */
#define CPG_PARAM_RING 8

/* Launch-shape candidates of the online tuner: solve block size and
 * whether the tree step may stage node pools in shared memory. */
#define CPG_TUNE_CANDIDATES 6
#define CPG_TUNE_ROUNDS 2
#define CPG_TUNE_PERIOD 256
#define CPG_TUNE_FIRST 32
static const int tune_threads[CPG_TUNE_CANDIDATES] = { 64, 128, 256, 64, 128, 256 };
static const int tune_tree[CPG_TUNE_CANDIDATES] = { -1, -1, -1, 0, 0, 0 };

struct DevSet {
	cpgSet d;                 /* device pointers; counts valid on host too */
	cpgWorld *hworld;
	cpgParams *hparams;       /* pinned, CPG_PARAM_RING slots of nspaces each */
	cudaEvent_t paramEvent[CPG_PARAM_RING]; /* recorded after each slot's upload */
	int paramRecorded[CPG_PARAM_RING];
	int paramSlot;
	int *hstats;              /* pinned */
	double *hbodies;          /* pinned staging for body downloads */
	cudaEvent_t statsEvent;
	int statsPending;
	int stepsSinceCheck;      /* steps enqueued since the stats were last read */
	cpSpace **spaces;
	int nspaces;
	void *slab;
	size_t slabBytes;
	void *scratch;            /* per-step scratch outside the slab (not checkpointed) */
	cpgArb *gather;           /* arbiter snapshot staging */
	int *bridgeBuf;           /* collision handlers: separated slots (arbCap + 1 ints), slot lists */
	int bridgeCap;
	int gatherCap;
	int structStale;          /* the staging block holds body state the body structs do not have yet */
	unsigned long long pullGen; /* id of the download in the staging block (unique across sets) */
	size_t hstride;           /* doubles between two arrays of the staging block */
	void *graph;              /* the step's launches as a CUDA graph (cpgStepGraph) */
	int useGraph;             /* this call's steps replay the graph */
	long long stepCount;      /* steps launched */
	/* online tuning of many-world sets (launch shapes that give the same
	 * results): candidates timed on interleaved steps, then the fastest */
	long long tuneNext;       /* step at which the next tuning window opens */
	int tuneIdx;              /* position in the open window */
	double tuneMs[CPG_TUNE_CANDIDATES];
	int tuneBest;             /* chosen candidate, -1 before the first window */
	void *qbuf;               /* spatial queries: queries, hits, counts, status */
	size_t qbytes;
	double *bstates;          /* cpGpuSpaceGetBodyStates: device staging */
	int bstatesCap;
};


static cudaStream_t g_stream = NULL;
static int g_stream_user = 0;
static int g_timing = 0;
static int g_tree_stage = -1;
static int g_autotune = 1;
void cpGpuSetAutotune(int on) { g_autotune = on ? 1 : 0; }
static int g_rollout_record = 1;
void cpGpuDebugSetRolloutRecording(int on) { g_rollout_record = on ? 1 : 0; }
static int g_solve_threads = 0, g_solve_stage = -1, g_solve_layout = 0;
void cpGpuDebugSetSolveShape(int threads, int maxBodies)
{
	g_solve_threads = (threads == 32 || threads == 64 || threads == 128 || threads == 256 || threads == 512) ? threads : 0;
	g_solve_stage = maxBodies < 0 ? -1 : maxBodies;
}
void cpGpuDebugSetSolveLayout(int policy) { g_solve_layout = (policy >= 0 && policy <= 3) ? policy : 0; }
/* the coloured sweep by dataflow measured slower than with a grid barrier
 * per colour (0.77 against 0.51 ms on 20,000 settled circles), so it is
 * off unless asked for */
static int g_flow_solve = 0;
void cpGpuDebugSetFlowSolve(int on) { g_flow_solve = on ? 1 : 0; }
static int g_flow_spin = 0, g_flow_withhold = 0;
void cpGpuDebugSetFlowWaitLimit(int polls, int withhold)
{
	g_flow_spin = polls > 0 ? polls : 0;
	g_flow_withhold = withhold ? 1 : 0;
}
/* capacity overrides for tests of the overflow latches (0: the defaults) */
static int g_cap_pairs_per_shape = 0, g_cap_pairs_extra = -1, g_cap_arbs = 0, g_cap_nodes = 0;
void cpGpuDebugSetCapacities(int pairsPerShape, int pairsExtra, int arbiterSlots, int nodes)
{
	g_cap_pairs_per_shape = pairsPerShape > 0 ? pairsPerShape : 0;
	g_cap_pairs_extra = pairsExtra >= 0 ? pairsExtra : -1;
	g_cap_arbs = arbiterSlots > 0 ? arbiterSlots : 0;
	g_cap_nodes = nodes > 0 ? nodes : 0;
}
/* measured neutral on 20,000 settled circles (the solve lost 26 us of
 * barrier-bound levels, the velocity kernel gained 23 us of gathers), so
 * off unless asked for */
static int g_warm_gather = 0;
void cpGpuDebugSetWarmStartGather(int on) { g_warm_gather = on ? 1 : 0; }
/* marking of a single space's exact tree: -1 automatic (the parallel
 * phases from CPG_PAR_MARK_MIN dynamic shapes up, where they beat one
 * thread), 0 always serial, 1 always parallel */
static int g_par_mark = -1;
#define CPG_PAR_MARK_MIN 1024
void cpGpuDebugSetParallelMarking(int on) { g_par_mark = on < 0 ? -1 : (on ? 1 : 0); }
static int g_coop_blocks = 0;
/* At most n blocks in the cooperative kernels (0: one per SM): a launch
 * shape for measurements; every shape gives the same results. */
void cpGpuDebugSetCoopBlocks(int n) { g_coop_blocks = n > 0 ? n : 0; }
void cpGpuDebugSetTreeStaging(int maxNodes) { g_tree_stage = maxNodes < 0 ? -1 : maxNodes; }
static int g_whole_grid = 0;     /* 1: single-world sets always use the whole-grid solve */

static cudaStream_t lib_stream(void)
{
	if(!g_stream && !g_stream_user) cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking);
	return g_stream;
}

void cpGpuSetStream(void *stream) { g_stream = (cudaStream_t)stream; g_stream_user = (stream != NULL); }
void cpGpuSetTiming(int enabled) { g_timing = enabled; }
void cpGpuDebugSetWholeGridSolve(int always) { g_whole_grid = always ? 1 : 0; }
long long cpGpuGetLaunchCount(int reset) { return cpg_launch_count(reset); }

static const int kPrimes[] = {
	/* leaf-set table sizes (src/prime.h:25-55) */
	5, 13, 23, 47, 97, 193, 389, 769, 1543, 3079, 6151, 12289, 24593, 49157,
	98317, 196613, 393241, 786433, 1572869, 3145739, 6291469, 12582917,
	25165843, 50331653, 100663319, 201326611, 402653189, 805306457, 1610612741, 0,
};

static unsigned next_prime(unsigned n)
{
	int i = 0;
	while(n > (unsigned)kPrimes[i] && kPrimes[i + 1]) i++;
	return (unsigned)kPrimes[i];
}

/* Largest table size the leaf set reaches holding n leaves
 * (cpHashSet.c:81-85, 152-176: grow when entries >= size). */
static int bins_for(int n)
{
	unsigned size = next_prime(0);
	for(int e = 1; e <= n; e++) if((unsigned)e >= size) size = next_prime(size + 1);
	return (int)size;
}

typedef struct Layout {
	size_t off;
	size_t bytes;
} Layout;

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

/* Carve the set's arrays out of one device allocation. */
#define CARVE(field, type, count) do { \
	size_t bytes_ = align256(sizeof(type)*(size_t)((count) > 0 ? (count) : 1)); \
	if(pass) d->field = (type *)(base + total); \
	total += bytes_; \
} while(0)

static size_t carve_set(cpgSet *d, char *base, int pass)
{
	size_t total = 0;
	int W = d->nworlds, NB = d->totalBodies, NS = d->totalShapes, NV = d->totalVerts, NC = d->totalCons;
	CARVE(world, cpgWorld, W); CARVE(params, cpgParams, W); CARVE(tree, cpgTree, W);
	CARVE(px, double, NB); CARVE(py, double, NB); CARVE(vx, double, NB); CARVE(vy, double, NB);
	CARVE(fx, double, NB); CARVE(fy, double, NB); CARVE(ang, double, NB); CARVE(w, double, NB); CARVE(tq, double, NB);
	CARVE(ta, double, NB); CARVE(tb, double, NB); CARVE(tc, double, NB); CARVE(td, double, NB);
	CARVE(ttx, double, NB); CARVE(tty, double, NB);
	CARVE(vbx, double, NB); CARVE(vby, double, NB); CARVE(wb, double, NB);
	CARVE(m, double, NB); CARVE(minv, double, NB); CARVE(i, double, NB); CARVE(iinv, double, NB);
	CARVE(cogx, double, NB); CARVE(cogy, double, NB);
	CARVE(btype, int, NB); CARVE(bworld, int, NB); CARVE(partStart, int, NB); CARVE(partCount, int, NB);
	CARVE(parts, int, d->totalParts); CARVE(last, int, NB);
	CARVE(springStart, int, NB); CARVE(springCount, int, NB); CARVE(springs, int, d->totalSprings);
	CARVE(skind, int, NS); CARVE(sbody, int, NS); CARVE(sleaf, int, NS); CARVE(sworld, int, NS);
	CARVE(svoff, int, NS); CARVE(svcount, int, NS);
	CARVE(sr, double, NS);
	CARVE(s0x, double, NS); CARVE(s0y, double, NS); CARVE(s1x, double, NS); CARVE(s1y, double, NS);
	CARVE(snx, double, NS); CARVE(sny, double, NS);
	CARVE(w0x, double, NS); CARVE(w0y, double, NS); CARVE(w1x, double, NS); CARVE(w1y, double, NS);
	CARVE(wnx, double, NS); CARVE(wny, double, NS);
	CARVE(atx, double, NS); CARVE(aty, double, NS); CARVE(btx, double, NS); CARVE(bty, double, NS);
	CARVE(bbl, double, NS); CARVE(bbb, double, NS); CARVE(bbr, double, NS); CARVE(bbt, double, NS);
	CARVE(se, double, NS); CARVE(su, double, NS); CARVE(svx, double, NS); CARVE(svy, double, NS);
	CARVE(sgroup, unsigned long long, NS); CARVE(scat, unsigned, NS); CARVE(smask, unsigned, NS);
	CARVE(ssensor, unsigned char, NS); CARVE(shost, unsigned char, NS); CARVE(shash, unsigned long long, NS);
	CARVE(lvx, double, NV); CARVE(lvy, double, NV); CARVE(lnx, double, NV); CARVE(lny, double, NV);
	CARVE(gvx, double, NV); CARVE(gvy, double, NV); CARVE(gnx, double, NV); CARVE(gny, double, NV);
	CARVE(nodes, cpgNode, d->totalNodes); CARVE(pairs, cpgPair, d->totalPairs);
	CARVE(dbins, int, d->totalDBins); CARVE(sbins, int, d->totalSBins);
	CARVE(ops, cpgOp, d->totalOps);
	CARVE(cands, cpgCand, d->totalCands); CARVE(narrow, cpgNarrow, d->totalCands);
	CARVE(candArb, int, d->totalCands); CARVE(arbList, int, d->totalCands); CARVE(prevList, int, d->totalCands);
	CARVE(prevCount, int, W);
	CARVE(keys, unsigned long long, d->arbCap); CARVE(arbs, cpgArb, d->arbCap);
	CARVE(joints, cpgJoint, NC); CARVE(jbias, double, NC);
	CARVE(unitA, int, d->totalUnits); CARVE(unitB, int, d->totalUnits); CARVE(unitKey, int, d->totalUnits);
	CARVE(worldOrder, int, W);
	CARVE(unitLevel, int, d->totalUnits); CARVE(unitOrder, int, d->totalUnits);
	CARVE(levelStart, int, d->totalUnits + W);
	CARVE(rows, cpgRow, d->totalUnits);
	CARVE(pbody, double, 8*NB);
	CARVE(dynShapes, int, NS);
	CARVE(sortKA, unsigned, NS); CARVE(sortKB, unsigned, NS); CARVE(rkeys, unsigned, NS);
	CARVE(sapCount, unsigned, NS + 1);
	CARVE(rsHist, unsigned, 256*CPG_SORT_MAX_BLOCKS + 256);
	CARVE(sortK64, unsigned long long, NS);
	CARVE(sortVA, int, NS); CARVE(sortVB, int, NS);
	CARVE(claim, unsigned long long, NB); CARVE(cmask, unsigned long long, NB);
	CARVE(colorCursor, int, 512);
	CARVE(sapBB, long long, 4*NS);
	{
		/* the dataflow sweep runs on single-world sets only */
		int one = (W == 1);
		CARVE(flowPred, int, one ? 2*d->totalUnits : 1);
		CARVE(flowDone, int, one ? d->totalUnits : 1);
		CARVE(flowPos, int, one ? 64*NB : 1);
		/* the parallel marking's scratch: 9 arrays per node, 2 per pair
		 * slot, 2 incidences of 2 ints per pair slot, block sums */
		size_t nn1 = (size_t)d->totalNodes + 1, np1 = (size_t)d->totalPairs + 1;
		CARVE(markScratch, int, one ? (9*nn1 + 2*np1 + 4*(size_t)d->totalPairs + 1025) : 1);
	}
	CARVE(sapPart, float, 4*CPG_SORT_MAX_BLOCKS);
	CARVE(gcells, int, 2*d->numcells);
	CARVE(gbinHandle, int, 2*d->gbinCap); CARVE(gbinNext, int, 2*d->gbinCap);
	CARVE(stats, int, 16);
	return total;
}

static int body_type_(const cpBody *b)
{
	/* cpBody.c:136-146 */
	if(b->idleTime == INF_) return CP_BODY_TYPE_STATIC;
	if(b->m == INF_) return CP_BODY_TYPE_KINEMATIC;
	return CP_BODY_TYPE_DYNAMIC;
}

/* Host staging helpers */
#define HALLOC(type, n) ((type *)calloc((size_t)((n) > 0 ? (n) : 1), sizeof(type)))

static int h2d(void *dst, const void *src, size_t bytes)
{
	if(bytes == 0) return 1;
	return cuda_ok(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, lib_stream()), "upload");
}

static int d2h(void *dst, const void *src, size_t bytes)
{
	if(bytes == 0) return 1;
	return cuda_ok(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, lib_stream()), "download");
}

/* A world's bodies on the device: the dynamic array (awake dynamic and
 * kinematic bodies), the sleeping bodies, the static array, the space's
 * static body. */
static int world_body_count(const cpSpace *sp) { return sp->ndyn + sp->nslp + sp->nstat + 1; }

static cpBody *world_body(cpSpace *sp, int i)
{
	if(i < sp->ndyn) return sp->dyn[i];
	i -= sp->ndyn;
	if(i < sp->nslp) return sp->slp[i];
	i -= sp->nslp;
	if(i < sp->nstat) return sp->stat[i];
	return &sp->staticBody;
}

/* Upload the mutable state of every body of world w. */
static int upload_bodies(DevSet *ds, int w)
{
	cpSpace *sp = ds->spaces[w];
	cpgSet *d = &ds->d;
	int n = world_body_count(sp), off = ds->hworld[w].bodyOff;
	double *buf = HALLOC(double, 24*n);
	double *f[24];
	for(int k = 0; k < 24; k++) f[k] = buf + (size_t)k*n;
	for(int i = 0; i < n; i++){
		cpBody *b = world_body(sp, i);
		b->index = i;
		b->devOwner = ds;
		f[0][i] = b->p.x; f[1][i] = b->p.y; f[2][i] = b->v.x; f[3][i] = b->v.y;
		f[4][i] = b->f.x; f[5][i] = b->f.y; f[6][i] = b->a; f[7][i] = b->w; f[8][i] = b->t;
		f[9][i] = b->transform.a; f[10][i] = b->transform.b; f[11][i] = b->transform.c; f[12][i] = b->transform.d;
		f[13][i] = b->transform.tx; f[14][i] = b->transform.ty;
		f[15][i] = b->v_bias.x; f[16][i] = b->v_bias.y; f[17][i] = b->w_bias;
		f[18][i] = b->m; f[19][i] = b->m_inv; f[20][i] = b->i; f[21][i] = b->i_inv;
		f[22][i] = b->cog.x; f[23][i] = b->cog.y;
	}
	double *dst[24] = { d->px, d->py, d->vx, d->vy, d->fx, d->fy, d->ang, d->w, d->tq,
		d->ta, d->tb, d->tc, d->td, d->ttx, d->tty, d->vbx, d->vby, d->wb,
		d->m, d->minv, d->i, d->iinv, d->cogx, d->cogy };
	int ok = 1;
	for(int k = 0; k < 24; k++) ok &= h2d(dst[k] + off, f[k], sizeof(double)*(size_t)n);
	cudaStreamSynchronize(lib_stream());
	free(buf);
	return ok;
}

/* The bodies' device state into the pinned staging block.  Returns 0 when
 * it could not be brought. */
static int download_bodies_raw(DevSet *ds)
{
	cpgSet *d = &ds->d;
	int NB = d->totalBodies;
	/* px .. wb are carved back to back (each padded to 256 bytes), so one
	 * copy into the pinned staging block brings all eighteen arrays */
	size_t stride = (size_t)(d->py - d->px);
	size_t bytes = (size_t)((char *)(d->wb + NB) - (char *)d->px);
	if(!ds->hbodies){
		if(!cuda_ok(cudaMallocHost((void **)&ds->hbodies, 18*stride*sizeof(double)), "cudaMallocHost")){ ds->hbodies = NULL; return 0; }
	}
	ds->hstride = stride;
	const double *src[18] = { d->px, d->py, d->vx, d->vy, d->fx, d->fy, d->ang, d->w, d->tq,
		d->ta, d->tb, d->tc, d->td, d->ttx, d->tty, d->vbx, d->vby, d->wb };
	int contiguous = 1;
	for(int k = 0; k < 18; k++) contiguous &= (src[k] == d->px + (size_t)k*stride);
	if(contiguous){
		if(!d2h(ds->hbodies, d->px, bytes)) return 0;
	} else {
		for(int k = 0; k < 18; k++) if(!d2h(ds->hbodies + (size_t)k*stride, src[k], sizeof(double)*(size_t)NB)) return 0;
	}
	return cuda_ok(cudaStreamSynchronize(lib_stream()), "download bodies");
}

/* The staging block into the dynamic bodies' structs. */
static void unpack_bodies(DevSet *ds)
{
	if(!ds->hbodies) return;
	size_t stride = ds->hstride;
	const double *f[18];
	for(int k = 0; k < 18; k++) f[k] = ds->hbodies + (size_t)k*stride;
	for(int w = 0; w < ds->nspaces; w++){
		cpSpace *sp = ds->spaces[w];
		int off = ds->hworld[w].bodyOff;
		for(int i = 0; i < sp->ndyn; i++){
			cpBody *b = sp->dyn[i];
			int g = off + i;
			b->p = cpv(f[0][g], f[1][g]); b->v = cpv(f[2][g], f[3][g]); b->f = cpv(f[4][g], f[5][g]);
			b->a = f[6][g]; b->w = f[7][g]; b->t = f[8][g];
			b->transform = cpTransformNew(f[9][g], f[10][g], f[11][g], f[12][g], f[13][g], f[14][g]);
			b->v_bias = cpv(f[15][g], f[16][g]); b->w_bias = f[17][g];
			b->pullGen = ds->pullGen;
		}
	}
}

/* One body's state from the staging block: a getter that reads every body
 * after a step touches each struct once, instead of a pass that unpacks
 * them all and a second pass that reads them. */
static int unpack_one(DevSet *ds, cpSpace *sp, cpBody *b)
{
	int i = b->index;
	if(!ds->hbodies || i < 0 || i >= sp->ndyn || sp->dyn[i] != b) return 0;
	size_t stride = ds->hstride;
	const double *f = ds->hbodies + ds->hworld[sp->world].bodyOff + i;
	b->p = cpv(f[0], f[stride]); b->v = cpv(f[2*stride], f[3*stride]); b->f = cpv(f[4*stride], f[5*stride]);
	b->a = f[6*stride]; b->w = f[7*stride]; b->t = f[8*stride];
	b->transform = cpTransformNew(f[9*stride], f[10*stride], f[11*stride], f[12*stride], f[13*stride], f[14*stride]);
	b->v_bias = cpv(f[15*stride], f[16*stride]); b->w_bias = f[17*stride];
	b->pullGen = ds->pullGen;
	return 1;
}

/* Whether a shape's arbiters need the host's callbacks: the default
 * handler was asked for, or its collision type has a handler of its own
 * (typed or wildcard).  Others meet only do-nothing handlers, whose rule
 * the device applies itself. */
static int shape_needs_host_(const cpSpace *sp, const cpShape *s)
{
	if(!sp->handlersOn) return 0;
	if(sp->defaultTouched) return 1;
	for(int i = 0; i < sp->nhandlers; i++){
		const cpCollisionHandler *h = sp->handlers[i];
		if(h->typeA == s->ctype || h->typeB == s->ctype) return 1;
	}
	return 0;
}

static int upload_shapes(DevSet *ds, int w)
{
	cpSpace *sp = ds->spaces[w];
	cpgSet *d = &ds->d;
	int n = sp->nshapes, off = ds->hworld[w].shapeOff;
	double *buf = HALLOC(double, 30*n);
	double *f[30];
	for(int k = 0; k < 30; k++) f[k] = buf + (size_t)k*n;
	int *ib = HALLOC(int, 5*n);
	int *kind = ib, *body = ib + n, *voff = ib + 2*n, *vcount = ib + 3*n, *wld = ib + 4*n;
	unsigned long long *grp = HALLOC(unsigned long long, 2*n), *hsh = grp + n;
	unsigned *cm = HALLOC(unsigned, 2*n), *cat = cm, *msk = cm + n;
	unsigned char *sens = HALLOC(unsigned char, n);
	unsigned char *hflag = HALLOC(unsigned char, n);
	int nv = 0;
	int staticIndex = world_body_count(sp) - 1;
	for(int i = 0; i < n; i++){
		cpShape *s = sp->shapes[i];
		if(!s){
			/* the slot of a removed shape: on the space's static body, in no
			 * index, so no kernel reads it (buffers are zeroed) */
			kind[i] = CPG_CIRCLE; body[i] = staticIndex; wld[i] = w;
			hsh[i] = (unsigned long long)i; voff[i] = nv; vcount[i] = 0;
			continue;
		}
		kind[i] = s->kind; body[i] = s->body->index; wld[i] = w;
		f[0][i] = s->r;
		cpVect l0 = s->kind == CPG_CIRCLE ? s->c : s->sa, l1 = s->sb, ln = s->sn;
		cpVect g0 = s->kind == CPG_CIRCLE ? s->tc : s->ta, g1 = s->tb, gn = s->tn;
		f[1][i] = l0.x; f[2][i] = l0.y; f[3][i] = l1.x; f[4][i] = l1.y; f[5][i] = ln.x; f[6][i] = ln.y;
		f[7][i] = g0.x; f[8][i] = g0.y; f[9][i] = g1.x; f[10][i] = g1.y; f[11][i] = gn.x; f[12][i] = gn.y;
		f[13][i] = s->a_tangent.x; f[14][i] = s->a_tangent.y; f[15][i] = s->b_tangent.x; f[16][i] = s->b_tangent.y;
		f[17][i] = s->bb.l; f[18][i] = s->bb.b; f[19][i] = s->bb.r; f[20][i] = s->bb.t;
		f[21][i] = s->e; f[22][i] = s->u; f[23][i] = s->surfaceV.x; f[24][i] = s->surfaceV.y;
		grp[i] = (unsigned long long)s->filter.group; cat[i] = s->filter.categories; msk[i] = s->filter.mask;
		sens[i] = s->sensor; hsh[i] = (unsigned long long)s->hashid;
		hflag[i] = (unsigned char)shape_needs_host_(sp, s);
		voff[i] = nv; vcount[i] = s->count;
		nv += s->count;
	}
	double *vb = HALLOC(double, 8*nv);
	for(int i = 0, k = 0; i < n; i++){
		cpShape *s = sp->shapes[i];
		if(!s) continue;
		for(int j = 0; j < s->count; j++, k++){
			vb[k] = s->lv[j].x; vb[nv + k] = s->lv[j].y; vb[2*nv + k] = s->ln[j].x; vb[3*nv + k] = s->ln[j].y;
			vb[4*nv + k] = s->gv[j].x; vb[5*nv + k] = s->gv[j].y; vb[6*nv + k] = s->gn[j].x; vb[7*nv + k] = s->gn[j].y;
		}
	}
	int ok = 1;
	size_t DB = sizeof(double)*(size_t)n, IB = sizeof(int)*(size_t)n;
	ok &= h2d(d->skind + off, kind, IB); ok &= h2d(d->sbody + off, body, IB); ok &= h2d(d->sworld + off, wld, IB);
	ok &= h2d(d->svoff + off, voff, IB); ok &= h2d(d->svcount + off, vcount, IB);
	double *dst[25] = { d->sr, d->s0x, d->s0y, d->s1x, d->s1y, d->snx, d->sny, d->w0x, d->w0y, d->w1x, d->w1y,
		d->wnx, d->wny, d->atx, d->aty, d->btx, d->bty, d->bbl, d->bbb, d->bbr, d->bbt, d->se, d->su, d->svx, d->svy };
	for(int k = 0; k < 25; k++) ok &= h2d(dst[k] + off, f[k], DB);
	ok &= h2d(d->sgroup + off, grp, sizeof(unsigned long long)*(size_t)n);
	ok &= h2d(d->shash + off, hsh, sizeof(unsigned long long)*(size_t)n);
	ok &= h2d(d->scat + off, cat, sizeof(unsigned)*(size_t)n);
	ok &= h2d(d->smask + off, msk, sizeof(unsigned)*(size_t)n);
	ok &= h2d(d->ssensor + off, sens, (size_t)n);
	ok &= h2d(d->shost + off, hflag, (size_t)n);
	int voffw = ds->hworld[w].vertOff;
	double *vdst[8] = { d->lvx, d->lvy, d->lnx, d->lny, d->gvx, d->gvy, d->gnx, d->gny };
	for(int k = 0; k < 8; k++) ok &= h2d(vdst[k] + voffw, vb + (size_t)k*nv, sizeof(double)*(size_t)nv);
	cudaStreamSynchronize(lib_stream());
	free(buf); free(ib); free(grp); free(cm); free(sens); free(hflag); free(vb);
	return ok;
}

static int upload_joints(DevSet *ds, int w, int params_only)
{
	cpSpace *sp = ds->spaces[w];
	cpgSet *d = &ds->d;
	int n = sp->ncons, off = ds->hworld[w].consOff;
	if(n == 0) return 1;
	int ok = 1;
	if(!params_only){
		cpgJoint *rec = HALLOC(cpgJoint, n);
		for(int i = 0; i < n; i++){
			cpConstraint *c = sp->cons[i];
			cpgJoint *j = &rec[i];
			*j = c->rec;
			j->kind = c->kind; j->a = c->a->index; j->b = c->b->index;
			j->ax = c->anchorA.x; j->ay = c->anchorA.y; j->bx = c->anchorB.x; j->by = c->anchorB.y;
			j->maxForce = c->maxForce; j->maxBias = c->maxBias;
			j->dist = c->dist; j->min = c->min; j->max = c->max;
			j->gax = c->grv_a.x; j->gay = c->grv_a.y; j->gbx = c->grv_b.x; j->gby = c->grv_b.y;
			j->gnx = c->grv_n.x; j->gny = c->grv_n.y;
			j->restLength = (c->kind == CPG_DRSPRING) ? c->restAngle : c->restLength;
			j->stiffness = c->stiffness; j->damping = c->damping;
			j->phase = c->phase; j->ratchet = c->ratchet; j->ratio = c->ratio; j->ratioInv = c->ratio_inv; j->rate = c->rate;
		}
		ok &= h2d(d->joints + off, rec, sizeof(cpgJoint)*(size_t)n);
		cudaStreamSynchronize(lib_stream());
		free(rec);
	}
	return ok;
}

/* Joint bias terms 1 - pow(errorBias, dt) (chipmunk_private.h:265-268),
 * evaluated on the host so they round like the reference's libm call. */
static int upload_joint_bias(DevSet *ds, int w, double dt)
{
	cpSpace *sp = ds->spaces[w];
	int n = sp->ncons;
	if(n == 0) return 1;
	double *b = HALLOC(double, n);
	double lastE = 0.0, lastV = 0.0; int have = 0;
	for(int i = 0; i < n; i++){
		double e = sp->cons[i]->errorBias;
		if(!have || e != lastE){ lastE = e; lastV = 1.0 - pow(e, dt); have = 1; }
		b[i] = lastV;
	}
	int ok = h2d(ds->d.jbias + ds->hworld[w].consOff, b, sizeof(double)*(size_t)n);
	cudaStreamSynchronize(lib_stream());
	free(b);
	return ok;
}

static void devset_free(DevSet *ds)
{
	if(!ds) return;
	if(ds->slab) cudaFree(ds->slab);
	if(ds->scratch) cudaFree(ds->scratch);
	if(ds->graph) cpg_step_graph_free(ds->graph);
	if(ds->gather) cudaFree(ds->gather);
	if(ds->bridgeBuf) cudaFree(ds->bridgeBuf);
	if(ds->qbuf) cudaFree(ds->qbuf);
	if(ds->bstates) cudaFree(ds->bstates);
	if(ds->hparams) cudaFreeHost(ds->hparams);
	if(ds->hstats) cudaFreeHost(ds->hstats);
	if(ds->hbodies) cudaFreeHost(ds->hbodies);
	if(ds->statsEvent) cudaEventDestroy(ds->statsEvent);
	for(int i = 0; i < CPG_PARAM_RING; i++) if(ds->paramEvent[i]) cudaEventDestroy(ds->paramEvent[i]);
	for(int w = 0; w < ds->nspaces; w++){
		if(ds->spaces[w]->dev == ds){ ds->spaces[w]->dev = NULL; }
	}
	free(ds->hworld);
	free(ds->spaces);
	free(ds);
}

static int device_available(void)
{
	static int ready = 0;
	int n = 0;
	if(cudaGetDeviceCount(&n) != cudaSuccess || n == 0){
		set_error(CP_GPU_ERR_NO_DEVICE, "no CUDA device is visible");
		return 0;
	}
	if(!ready){
		/* the narrow phase keeps the EPA hull (about 4 KB) on the stack */
		cuda_ok(cudaDeviceSetLimit(cudaLimitStackSize, 8192), "stack limit");
		ready = 1;
	}
	return 1;
}

/* Build a device set holding `spaces` (each becomes one world).  With
 * `from` (a single space's previous set), the tree, pair cache, leaf sets
 * and arbiter cache carry over from it instead of starting empty, and the
 * index edits recorded since it was built replay on top. */
static DevSet *devset_build(cpSpace **spaces, int nspaces, DevSet *from)
{
	if(!device_available()) return NULL;
	DevSet *ds = (DevSet *)calloc(1, sizeof(DevSet));
	ds->nspaces = nspaces;
	ds->spaces = (cpSpace **)malloc(sizeof(cpSpace *)*(size_t)nspaces);
	memcpy(ds->spaces, spaces, sizeof(cpSpace *)*(size_t)nspaces);
	ds->hworld = HALLOC(cpgWorld, nspaces);
	cpgSet *d = &ds->d;
	d->nworlds = nspaces;
	long long NB = 0, NS = 0, NV = 0, NC = 0, NN = 0, NP = 0, NDB = 0, NSB = 0, NCD = 0, NU = 0, NO = 0, NPT = 0, NSP = 0;
	for(int w = 0; w < nspaces; w++){
		cpSpace *sp = spaces[w];
		cpgWorld *W = &ds->hworld[w];
		int nb = world_body_count(sp);
		int nverts = 0, ndynShapes = 0, nstatShapes = 0;
		for(int i = 0; i < sp->nshapes; i++){
			cpShape *s = sp->shapes[i];
			if(!s) continue;
			nverts += s->count;
			if(body_type_(s->body) == CP_BODY_TYPE_STATIC) nstatShapes++; else ndynShapes++;
		}
		int nparts = 0, nsprings = 0;
		for(int i = 0; i < sp->ncons; i++){
			if(!sp->cons[i]->collideBodies) nparts += 2;
			if(sp->cons[i]->kind == CPG_DSPRING || sp->cons[i]->kind == CPG_DRSPRING) nsprings += 2;
		}
		W->bodyOff = (int)NB; W->nbodies = nb; W->ndyn = sp->ndyn;
		W->shapeOff = (int)NS; W->nshapes = sp->nshapes;
		W->vertOff = (int)NV; W->nverts = nverts;
		W->consOff = (int)NC; W->ncons = sp->ncons;
		/* capacities by shape slots (removed shapes keep theirs), so a set
		 * rebuilt after removals holds at least what its predecessor held */
		int churn = (sp->nshapes != ndynShapes + nstatShapes) || from || sp->nslp > 0;
		W->nodeOff = (int)NN; W->nodeCap = 2*sp->nshapes + 4;
		W->pairOff = (int)NP; W->pairCap = 16*sp->nshapes + 256;
		if(g_cap_pairs_per_shape || g_cap_pairs_extra >= 0)
			W->pairCap = (g_cap_pairs_per_shape ? g_cap_pairs_per_shape : 16)*sp->nshapes + (g_cap_pairs_extra >= 0 ? g_cap_pairs_extra : 256);
		if(g_cap_nodes && g_cap_nodes < W->nodeCap) W->nodeCap = g_cap_nodes;
		W->dbinOff = (int)NDB; W->dbinCap = bins_for(churn ? sp->nshapes : ndynShapes);
		W->sbinOff = (int)NSB; W->sbinCap = bins_for(churn ? sp->nshapes : nstatShapes);
		if(from){
			/* never below the predecessor's pools, whose contents move over */
			const cpgWorld *O = &from->hworld[0];
			if(W->nodeCap < O->nodeCap) W->nodeCap = O->nodeCap;
			if(W->pairCap < O->pairCap) W->pairCap = O->pairCap;
			if(W->dbinCap < O->dbinCap) W->dbinCap = O->dbinCap;
			if(W->sbinCap < O->sbinCap) W->sbinCap = O->sbinCap;
		}
		W->candOff = (int)NCD; W->candCap = W->pairCap;
		W->unitOff = (int)NU; W->unitCap = W->candCap + sp->ncons;
		W->opOff = (int)NO; W->nops = sp->nops;
		W->partOff = (int)NPT;
		W->springOff = (int)NSP;
		W->dynShapeOff = (int)NS; W->ndynShapes = ndynShapes;
		NB += nb; NS += sp->nshapes; NV += nverts; NC += sp->ncons;
		NN += W->nodeCap; NP += W->pairCap; NDB += W->dbinCap; NSB += W->sbinCap;
		NCD += W->candCap; NU += W->unitCap; NO += sp->nops; NPT += nparts; NSP += nsprings;
	}
	if(NB > 0x7fffffffLL || NCD > 0x7fffffffLL || NU > 0x7fffffffLL){
		set_error(CP_GPU_ERR_OVERFLOW, "set too large");
		devset_free(ds);
		return NULL;
	}
	d->totalBodies = (int)NB; d->totalShapes = (int)NS; d->totalVerts = (int)NV; d->totalCons = (int)NC;
	d->totalNodes = (int)NN; d->totalPairs = (int)NP; d->totalDBins = (int)NDB; d->totalSBins = (int)NSB;
	d->totalCands = (int)NCD; d->totalUnits = (int)NU; d->totalOps = (int)NO; d->totalParts = (int)NPT;
	d->totalSprings = (int)NSP;
	long long arbCap = 1024;
	while(arbCap < 8*NS + 1024) arbCap *= 2;
	if(g_cap_arbs){ arbCap = 1; while(arbCap < g_cap_arbs) arbCap *= 2; }
	if(from && arbCap < from->d.arbCap) arbCap = from->d.arbCap;
	d->arbCap = (int)arbCap;
	/* a single space on the spatial hash: its grids and bin pools, the
	 * pools sized from the shapes' boxes now with room to grow */
	d->useHash = 0; d->numcells = 0; d->gbinCap = 0; d->celldim = 0.0;
	if(nspaces == 1 && spaces[0]->useHash){
		cpSpace *sp = spaces[0];
		d->useHash = 1;
		d->numcells = sp->hashCells;
		d->celldim = sp->hashDim;
		long long bins = 0;
		for(int i = 0; i < sp->nshapes; i++){
			cpShape *sh = sp->shapes[i];
			if(!sh) continue;
			double w = floor(sh->bb.r/sp->hashDim) - floor(sh->bb.l/sp->hashDim) + 1.0;
			double h = floor(sh->bb.t/sp->hashDim) - floor(sh->bb.b/sp->hashDim) + 1.0;
			double cells = (w > 0.0 && h > 0.0) ? w*h : 1.0;
			bins += cells < (double)sp->hashCells ? (long long)cells : sp->hashCells;
		}
		long long cap = 4*bins + 16LL*sp->nshapes + 1024;
		if(from && from->d.useHash && cap < from->d.gbinCap) cap = from->d.gbinCap;
		if(cap > 0x3fffffffLL) cap = 0x3fffffffLL;
		d->gbinCap = (int)cap;
	}

	size_t bytes = carve_set(d, NULL, 0);
	ds->slabBytes = bytes;
	if(!cuda_ok(cudaMalloc(&ds->slab, bytes), "cudaMalloc set")){ devset_free(ds); return NULL; }
	carve_set(d, (char *)ds->slab, 1);
	/* per-step scratch that no checkpoint needs: its own allocation */
	{
		size_t nb = sizeof(int)*(size_t)CPG_PAIR_TYPES*(size_t)(d->totalCands > 0 ? d->totalCands : 1);
		if(!cuda_ok(cudaMalloc(&ds->scratch, nb + 256), "cudaMalloc narrow scratch")){ devset_free(ds); return NULL; }
		d->nbCount = (int *)ds->scratch;
		d->nbucket = (int *)((char *)ds->scratch + 256);
	}
	cudaStream_t st = lib_stream();
	int ok = 1;
	ok &= cuda_ok(cudaMemsetAsync(ds->slab, 0, bytes, st), "memset set");
	ok &= cuda_ok(cudaMemsetAsync(d->dbins, 0xff, sizeof(int)*(size_t)(NDB > 0 ? NDB : 1), st), "memset bins");
	ok &= cuda_ok(cudaMemsetAsync(d->sbins, 0xff, sizeof(int)*(size_t)(NSB > 0 ? NSB : 1), st), "memset bins");
	if(d->useHash) ok &= cuda_ok(cudaMemsetAsync(d->gcells, 0xff, sizeof(int)*2*(size_t)d->numcells, st), "memset cells");
	ok &= cuda_ok(cudaMallocHost((void **)&ds->hparams, sizeof(cpgParams)*(size_t)nspaces*CPG_PARAM_RING), "cudaMallocHost");
	if(ok) memset(ds->hparams, 0, sizeof(cpgParams)*(size_t)nspaces*CPG_PARAM_RING);
	for(int i = 0; i < CPG_PARAM_RING && ok; i++) ok &= cuda_ok(cudaEventCreateWithFlags(&ds->paramEvent[i], cudaEventDisableTiming), "event");
	ok &= cuda_ok(cudaMallocHost((void **)&ds->hstats, sizeof(int)*16), "cudaMallocHost");
	ok &= cuda_ok(cudaEventCreateWithFlags(&ds->statsEvent, cudaEventDisableTiming), "event");
	if(!ok){ devset_free(ds); return NULL; }

	ok &= h2d(d->world, ds->hworld, sizeof(cpgWorld)*(size_t)nspaces);
	/* bodies of the predecessor set by their new index (read before the
	 * uploads below renumber them) */
	int *bodyMap = NULL;
	if(from){
		int oldNB = from->hworld[0].nbodies;
		bodyMap = HALLOC(int, oldNB);
		for(int i = 0; i < oldNB; i++) bodyMap[i] = -1;
		cpSpace *sp = spaces[0];
		int nb = world_body_count(sp);
		for(int i = 0; i < nb; i++){
			cpBody *b = world_body(sp, i);
			if(b->devOwner == from && b->index >= 0 && b->index < oldNB) bodyMap[b->index] = i;
		}
	}
	cpgTree *trees = HALLOC(cpgTree, nspaces);
	for(int w = 0; w < nspaces; w++){
		cpgTree *T = &trees[w];
		T->dynRoot = -1; T->statRoot = -1; T->treeStamp = 0;
		T->gbinTop[0] = T->gbinTop[1] = 0; T->gbinFree[0] = T->gbinFree[1] = -1;
		T->gstamp[0] = T->gstamp[1] = 1;
		T->freeNode = -1; T->freePair = -1;
		T->dynSize = next_prime(0); T->statSize = next_prime(0);
	}
	ok &= h2d(d->tree, trees, sizeof(cpgTree)*(size_t)nspaces);
	cudaStreamSynchronize(st);
	free(trees);

	for(int w = 0; w < nspaces; w++){
		cpSpace *sp = spaces[w];
		sp->dev = ds; sp->world = w;
		ok &= upload_bodies(ds, w);
		ok &= upload_shapes(ds, w);
		ok &= upload_joints(ds, w, 0);
		/* body -> world, type; partners with collideBodies off */
		cpgWorld *W = &ds->hworld[w];
		int nb = W->nbodies;
		int *bi = HALLOC(int, 4*nb);
		int *bw = bi, *bt = bi + nb, *pstart = bi + 2*nb, *pcount = bi + 3*nb;
		for(int i = 0; i < nb; i++){
			cpBody *b = world_body(sp, i);
			bw[i] = w;
			int t = body_type_(b);
			bt[i] = (t == CP_BODY_TYPE_STATIC) ? CPG_STATIC : (t == CP_BODY_TYPE_KINEMATIC ? CPG_KINEMATIC : CPG_DYNAMIC);
		}
		int np = 0;
		for(int i = 0; i < sp->ncons; i++) if(!sp->cons[i]->collideBodies){ pcount[sp->cons[i]->a->index]++; pcount[sp->cons[i]->b->index]++; np += 2; }
		for(int i = 0, acc = 0; i < nb; i++){ pstart[i] = acc; acc += pcount[i]; pcount[i] = 0; }
		int *parts = HALLOC(int, np);
		for(int i = 0; i < sp->ncons; i++){
			cpConstraint *c = sp->cons[i];
			if(c->collideBodies) continue;
			int a = c->a->index, b = c->b->index;
			parts[pstart[a] + pcount[a]++] = b;
			parts[pstart[b] + pcount[b]++] = a;
		}
		ok &= h2d(d->bworld + W->bodyOff, bw, sizeof(int)*(size_t)nb);
		ok &= h2d(d->btype + W->bodyOff, bt, sizeof(int)*(size_t)nb);
		ok &= h2d(d->partStart + W->bodyOff, pstart, sizeof(int)*(size_t)nb);
		ok &= h2d(d->partCount + W->bodyOff, pcount, sizeof(int)*(size_t)nb);
		ok &= h2d(d->parts + W->partOff, parts, sizeof(int)*(size_t)np);
		/* the springs on each body, in constraint order */
		{
			int *ss = HALLOC(int, 2*nb), *sstart = ss, *scount = ss + nb;
			int nsp = 0;
			for(int i = 0; i < sp->ncons; i++){
				cpConstraint *c = sp->cons[i];
				if(c->kind != CPG_DSPRING && c->kind != CPG_DRSPRING) continue;
				scount[c->a->index]++; scount[c->b->index]++; nsp += 2;
			}
			for(int i = 0, acc = 0; i < nb; i++){ sstart[i] = acc; acc += scount[i]; scount[i] = 0; }
			int *sl = HALLOC(int, nsp);
			for(int i = 0; i < sp->ncons; i++){
				cpConstraint *c = sp->cons[i];
				if(c->kind != CPG_DSPRING && c->kind != CPG_DRSPRING) continue;
				int a = c->a->index, b = c->b->index;
				sl[sstart[a] + scount[a]++] = i;
				sl[sstart[b] + scount[b]++] = i;
			}
			ok &= h2d(d->springStart + W->bodyOff, sstart, sizeof(int)*(size_t)nb);
			ok &= h2d(d->springCount + W->bodyOff, scount, sizeof(int)*(size_t)nb);
			ok &= h2d(d->springs + W->springOff, sl, sizeof(int)*(size_t)nsp);
			cudaStreamSynchronize(st);
			free(ss); free(sl);
		}
		ok &= h2d(d->ops + W->opOff, sp->ops, sizeof(cpgOp)*(size_t)sp->nops);
		int *dyns = HALLOC(int, sp->nshapes);
		int nds = 0;
		for(int i = 0; i < sp->nshapes; i++) if(sp->shapes[i] && body_type_(sp->shapes[i]->body) != CP_BODY_TYPE_STATIC) dyns[nds++] = i;
		ok &= h2d(d->dynShapes + W->dynShapeOff, dyns, sizeof(int)*(size_t)nds);
		cudaStreamSynchronize(st);
		free(bi); free(parts); free(dyns);
		sp->builtBodies = world_body_count(sp); sp->builtShapes = sp->nshapes; sp->builtCons = sp->ncons;
		sp->bodyDirty = sp->shapeDirty = sp->consDirty = sp->structDirty = 0;
		sp->jointDt = 0.0;
	}
	if(!ok){ devset_free(ds); return NULL; }
	d->hostNdyn = ds->hworld[0].ndynShapes;
	d->hostUnitsHint = 0;
	d->hostMaxBodies = 0;
	d->hostMaxNodes = 0;
	d->hostTreeStage = -1;
	ds->tuneNext = CPG_TUNE_FIRST;
	ds->tuneBest = -1;
	d->hostSolveThreads = 0;
	d->hostSolveStage = -1;
	d->solveLayout = 0;
	for(int w = 0; w < nspaces; w++){
		if(ds->hworld[w].nbodies > d->hostMaxBodies) d->hostMaxBodies = ds->hworld[w].nbodies;
		if(ds->hworld[w].nodeCap > d->hostMaxNodes) d->hostMaxNodes = ds->hworld[w].nodeCap;
	}
	/* worlds by decreasing shape count: the serial tree step of the largest
	 * worlds starts first */
	{
		int *ord = HALLOC(int, nspaces);
		for(int w = 0; w < nspaces; w++) ord[w] = w;
		/* insertion sort by key, stable, descending (counting sort would also do) */
		for(int i = 1; i < nspaces; i++){
			int x = ord[i], k = i;
			while(k > 0 && ds->hworld[ord[k - 1]].nshapes < ds->hworld[x].nshapes){ ord[k] = ord[k - 1]; k--; }
			ord[k] = x;
		}
		h2d(d->worldOrder, ord, sizeof(int)*(size_t)nspaces);
		cudaStreamSynchronize(lib_stream());
		free(ord);
	}
	if(from){
		/* the predecessor's tree and arbiter cache, bodies renumbered and
		 * the arbiters of removed shapes dropped */
		cpSpace *sp = spaces[0];
		int oldNB = from->hworld[0].nbodies, oldNS = from->hworld[0].nshapes;
		size_t bm = align256(sizeof(int)*(size_t)(oldNB > 0 ? oldNB : 1));
		size_t dm = align256((size_t)(oldNS > 0 ? oldNS : 1));
		size_t sm = sizeof(int)*(size_t)from->d.arbCap;
		unsigned char *dead = HALLOC(unsigned char, oldNS);
		for(int i = 0; i < oldNS; i++) dead[i] = (i >= sp->nshapes || sp->shapes[i] == NULL);
		char *tmp = NULL;
		int tok = cuda_ok(cudaMalloc((void **)&tmp, bm + dm + sm), "cudaMalloc transfer");
		if(tok){
			tok &= h2d(tmp, bodyMap, sizeof(int)*(size_t)oldNB);
			tok &= h2d(tmp + bm, dead, (size_t)oldNS);
			tok &= (cpg_launch_transfer(d, &from->d, (const int *)tmp, (const unsigned char *)(tmp + bm), (int *)(tmp + bm + dm), st) == 0);
			tok &= cuda_ok(cudaStreamSynchronize(st), "transfer");
			cudaFree(tmp);
		}
		free(dead);
		if(!tok){ free(bodyMap); set_error(CP_GPU_ERR_CUDA, "device state transfer failed"); devset_free(ds); return NULL; }
	}
	free(bodyMap);
	/* replay the recorded index edits, then clear the logs */
	if(cpg_launch_apply_ops(d, st) != 0){ set_error(CP_GPU_ERR_CUDA, "apply_ops launch failed"); devset_free(ds); return NULL; }
	for(int w = 0; w < nspaces; w++){ ds->hworld[w].nops = 0; spaces[w]->nops = 0; }
	h2d(d->world, ds->hworld, sizeof(cpgWorld)*(size_t)nspaces);
	if(!cuda_ok(cudaStreamSynchronize(st), "build")){ devset_free(ds); return NULL; }
	return ds;
}

static void check_stats(DevSet *ds);
static void space_detach(cpSpace *sp);
static cpFloat default_spring_force_(cpConstraint *c, cpFloat dist);
static cpFloat default_spring_torque_(cpConstraint *c, cpFloat relativeAngle);

/* Downloads so far: identifies the state in a staging block. */
static unsigned long long g_pull_gen = 0;

/* After a step: the device's body state into the staging block (the body
 * structs are unpacked from it only when something needs them). */
static void space_download(cpSpace *sp)
{
	if(!sp || !sp->dev || !sp->hostStale) return;
	DevSet *ds = sp->dev;
	/* the copy queues behind the step; once it is done so are the stats */
	int ok = download_bodies_raw(ds);
	check_stats(ds);
	if(!ok) return;
	for(int w = 0; w < ds->nspaces; w++){
		cpSpace *o = ds->spaces[w];
		o->hostStale = 0;
		o->snapValid = 0;
	}
	ds->pullGen = ++g_pull_gen;
	ds->structStale = 1;
}

/* The bodies' current state into their structs. */
static void space_pull(cpSpace *sp)
{
	if(!sp || !sp->dev) return;
	space_download(sp);
	DevSet *ds = sp->dev;
	if(ds->structStale){
		unpack_bodies(ds);
		ds->structStale = 0;
	}
}

static void check_stats(DevSet *ds)
{
	if(!ds->statsPending) return;
	cudaEventSynchronize(ds->statsEvent);
	ds->statsPending = 0;
	ds->stepsSinceCheck = 0;
	int err = ds->hstats[0];
	/* whole-grid solve pays off when one sweep level is wide enough */
	int units = ds->hstats[5] + (ds->nspaces == 1 ? ds->spaces[0]->ncons : 0);
	int levels = ds->hstats[6] > 0 ? ds->hstats[6] : 1;
	ds->d.hostUnitsHint = (ds->nspaces == 1 && units/levels >= 64) ? units : 0;
	if(err & CPG_ERR_FLOW){
		set_error(CP_GPU_ERR_TIMEOUT, "coloured sweep: a dataflow wait gave up (flags 0x%x)", err);
	} else if(err){
		set_error(CP_GPU_ERR_OVERFLOW, "device table overflow (flags 0x%x): pairs %d/1000, nodes %d/1000, candidates %d/1000",
			err, ds->hstats[1], ds->hstats[2], ds->hstats[7]);
	}
}

/* Upload what the host changed in world w since the last step. */
static void devset_flush_space(DevSet *ds, int w)
{
	cpSpace *sp = ds->spaces[w];
	if(sp->bodyDirty){ upload_bodies(ds, w); sp->bodyDirty = 0; }
	if(sp->shapeDirty){ upload_shapes(ds, w); sp->shapeDirty = 0; }
	if(sp->consDirty){ upload_joints(ds, w, 0); sp->consDirty = 0; sp->jointDt = 0.0; }
}

/* One step of every world of the set with per-world dt. */
static int bridge_buf_(DevSet *ds, int n);

/* part 0: the whole step; 1: up to the arbiter list; 2: the rest of the
 * step begun by part 1 (a single space; its set may have been rebuilt in
 * between, so the parameters go up again without advancing the stamp);
 * 3: the arbiter filter of part 2; 4: the rest of part 2 after the filter;
 * 5: part 4 through the velocity update; 6: the rest of part 4; 7: part 1
 * through the position update; 8: the rest of part 1. */
static int devset_step_part(DevSet *ds, const double *dts, cpSpace **only, int part)
{
	cpgSet *d = &ds->d;
	/* The bookkeeping of a step (overflow flags, level counts) is read back
	 * asynchronously; waiting for it every step would stop the host from
	 * queueing the next step while the device runs this one.  It is checked
	 * every CPG_STATS_INTERVAL steps and whenever the host reads state. */
	if(ds->stepsSinceCheck >= CPG_STATS_INTERVAL) check_stats(ds);
	int slot = ds->paramSlot;
	ds->paramSlot = (slot + 1) % CPG_PARAM_RING;
	if(ds->paramRecorded[slot]) cudaEventSynchronize(ds->paramEvent[slot]);
	cpgParams *hp = ds->hparams + (size_t)slot*ds->nspaces;
	for(int w = 0; w < ds->nspaces; w++){
		cpSpace *sp = ds->spaces[w];
		cpgParams *P = &hp[w];
		if((only && *only != sp) || dts[w] == 0.0){ P->active = 0; continue; }
		devset_flush_space(ds, w);
		double dt = dts[w];
		/* cpSpaceStep.c:339-344, 384, 399, 407 */
		cpFloat prev_dt;
		if(part >= 2 && part != 7) prev_dt = sp->prevDt;
		else {
			sp->stamp++;
			prev_dt = sp->prevDt = sp->curr_dt;
			sp->curr_dt = dt;
		}
		if(sp->jointDt != dt){ upload_joint_bias(ds, w, dt); sp->jointDt = dt; }
		P->dt = dt;
		P->dt_coef = (prev_dt == 0.0 ? 0.0 : dt/prev_dt);
		P->damping = pow(sp->damping, dt);
		P->slop = sp->collisionSlop;
		P->biasCoef = 1.0 - pow(sp->collisionBias, dt);
		P->gx = sp->gravity.x; P->gy = sp->gravity.y;
		P->iterations = sp->iterations;
		P->stamp = sp->stamp;
		P->persistence = sp->collisionPersistence;
		P->active = 1;
		sp->hostStale = 1;
		sp->consStale = 1;
		sp->shapesStale = 1;
		sp->snapValid = 0;
	}
	cudaStream_t st = lib_stream();
	if(g_whole_grid) d->hostUnitsHint = 0x7fffffff;
	d->hostTreeStage = g_tree_stage;
	d->hostSolveThreads = g_solve_threads;
	d->hostSolveStage = g_solve_stage;
	d->solveLayout = g_solve_layout;
	d->flowSolve = g_flow_solve;
	d->flowSpin = g_flow_spin;
	d->flowWithhold = g_flow_withhold;
	d->warmGather = g_warm_gather;
	d->hostCoopBlocks = g_coop_blocks;
	d->parMark = g_par_mark >= 0 ? g_par_mark : (d->hostNdyn >= CPG_PAR_MARK_MIN);
	/* collision handlers: the separations of the filter go to the host */
	d->bridge = (ds->nspaces == 1 && ds->spaces[0]->handlersOn && part != 0);
	d->sepSlots = d->sepCount = NULL;
	if(d->bridge){
		if(!bridge_buf_(ds, d->arbCap + 1)) return -1;
		d->sepSlots = ds->bridgeBuf;
		d->sepCount = ds->bridgeBuf + d->arbCap;
	}
	/* launch shapes of many-world sets: the tuner's candidates on the steps
	 * of a tuning window, its choice after it (debug settings win) */
	int tuning = -1;
	if(ds->nspaces >= 152 && g_autotune && g_solve_threads == 0 && g_tree_stage < 0){
		if(ds->stepCount >= ds->tuneNext){
			/* candidates in palindromic order: every candidate's steps sit
			 * at the same mean time, so a workload that grows or settles
			 * does not favour the ones timed first */
			int i = ds->tuneIdx, r = i/CPG_TUNE_CANDIDATES, j = i % CPG_TUNE_CANDIDATES;
			tuning = (r & 1) ? CPG_TUNE_CANDIDATES - 1 - j : j;
			d->hostSolveThreads = tune_threads[tuning];
			d->hostTreeStage = tune_tree[tuning];
		} else if(ds->tuneBest >= 0){
			d->hostSolveThreads = tune_threads[ds->tuneBest];
			d->hostTreeStage = tune_tree[ds->tuneBest];
		}
	}
	if(!h2d(d->params, hp, sizeof(cpgParams)*(size_t)ds->nspaces)) return -1;
	cudaEventRecord(ds->paramEvent[slot], st);
	ds->paramRecorded[slot] = 1;
	float ms[8] = {0};
	int mode = ds->spaces[0]->mode;
	int timed = g_timing || tuning >= 0;
	int lrc;
	/* many-world sets launch no cooperative kernels and keep their launch
	 * arguments from step to step: their step replays as one CUDA graph */
	if(part != 0) lrc = cpg_launch_step_part(d, d, mode, st, NULL, part);
	else if(ds->useGraph && !timed && !d->tape.on && ds->nspaces > 1) lrc = cpg_launch_step_graph(d, mode, st, &ds->graph);
	else lrc = cpg_launch_step(d, d, mode, st, timed ? ms : NULL);
	if(lrc != 0){
		set_error(CP_GPU_ERR_CUDA, "step launch failed");
		return -1;
	}
	if(part == 1 || part == 3 || part == 5 || part == 7 || part == 8) return 0;
	if(g_timing) for(int w = 0; w < ds->nspaces; w++) memcpy(ds->spaces[w]->phaseMs, ms, sizeof(ms));
	if(tuning >= 0){
		ds->tuneMs[tuning] += (double)ms[1] + (double)ms[6];
		if(++ds->tuneIdx == CPG_TUNE_CANDIDATES*CPG_TUNE_ROUNDS){
			int best = 0;
			for(int c = 1; c < CPG_TUNE_CANDIDATES; c++) if(ds->tuneMs[c] < ds->tuneMs[best]) best = c;
			ds->tuneBest = best;
			for(int c = 0; c < CPG_TUNE_CANDIDATES; c++) ds->tuneMs[c] = 0.0;
			ds->tuneIdx = 0;
			ds->tuneNext = ds->stepCount + CPG_TUNE_PERIOD;
		}
	}
	ds->stepCount++;
	if(!ds->statsPending){
		cudaMemcpyAsync(ds->hstats, d->stats, sizeof(int)*16, cudaMemcpyDeviceToHost, st);
		cudaEventRecord(ds->statsEvent, st);
		ds->statsPending = 1;
	}
	ds->stepsSinceCheck++;
	return 0;
}

static int devset_step(DevSet *ds, const double *dts, cpSpace **only) { return devset_step_part(ds, dts, only, 0); }

static int sleep_mode_(const cpSpace *sp);
static cpCollisionHandler handler_do_nothing_;
static int handlers_collide_(cpSpace *sp);
static int handlers_separate_(cpSpace *sp);
static int handlers_post_solve_(cpSpace *sp);
static int sleep_apply_edits_(cpSpace *sp);
static void graph_start_(cpSpace *sp);
static void graph_stop_(cpSpace *sp);
static int sleep_sync_(cpSpace *sp, cpFloat dt);

static inline cpConstraint *cons_next_(cpConstraint *c, cpBody *b);

static int space_supported(cpSpace *sp)
{
	if(sleep_mode_(sp) && (sp->mode != CP_GPU_SOLVER_ORDERED || (sp->dev && !sp->ownsDev))){
		set_error(CP_GPU_ERR_UNSUPPORTED, "sleeping runs in the exact-order mode of a standalone space");
		return 0;
	}
	if(sp->useHash && (sp->mode != CP_GPU_SOLVER_ORDERED || (sp->dev && !sp->ownsDev))){
		set_error(CP_GPU_ERR_UNSUPPORTED, "the spatial hash runs in the exact-order mode of a standalone space");
		return 0;
	}
	if(sp->handlersOn && (sp->mode != CP_GPU_SOLVER_ORDERED || (sp->dev && !sp->ownsDev))){
		set_error(CP_GPU_ERR_UNSUPPORTED, "collision handlers run in the exact-order mode of a standalone space");
		return 0;
	}
	for(int i = 0; i < sp->ndyn; i++){
		cpBody *b = sp->dyn[i];
		if(b->velocity_func != cpBodyUpdateVelocity || b->position_func != cpBodyUpdatePosition){
			if(sp->mode != CP_GPU_SOLVER_ORDERED || (sp->dev && !sp->ownsDev)){
				set_error(CP_GPU_ERR_UNSUPPORTED, "custom velocity and position functions run in the exact-order mode of a standalone space");
				return 0;
			}
			for(cpConstraint *c = b->constraintList; b->velocity_func != cpBodyUpdateVelocity && c; c = cons_next_(c, b)){
				if(c->kind == CPG_DSPRING || c->kind == CPG_DRSPRING){
					set_error(CP_GPU_ERR_UNSUPPORTED, "a body with a custom velocity function cannot carry a damped spring");
					return 0;
				}
			}
		}
	}
	for(int i = 0; i < sp->ncons; i++){
		cpConstraint *c = sp->cons[i];
		if((c->preSolve || c->postSolve) && (sp->mode != CP_GPU_SOLVER_ORDERED || (sp->dev && !sp->ownsDev))){
			set_error(CP_GPU_ERR_UNSUPPORTED, "constraint pre/post-solve callbacks run in the exact-order mode of a standalone space");
			return 0;
		}
		if((c->kind == CPG_DSPRING && c->springForceFunc != (cpDampedSpringForceFunc)default_spring_force_) ||
		   (c->kind == CPG_DRSPRING && c->springTorqueFunc != (cpDampedRotarySpringTorqueFunc)default_spring_torque_)){
			set_error(CP_GPU_ERR_UNSUPPORTED, "custom spring force or torque functions are not run on the GPU");
			return 0;
		}
	}
	return 1;
}

static int space_structure_changed(cpSpace *sp)
{
	return sp->dev && (world_body_count(sp) != sp->builtBodies || sp->nshapes != sp->builtShapes || sp->ncons != sp->builtCons);
}

/* cpSpaceStep.c:335-445 */
/* A space's own device set, current with the host's structure: built at
 * first use; rebuilt when objects were added or removed since, the host
 * holding the whole state (space_detach), carrying the device tree and
 * arbiter cache over and replaying the index edits recorded since, in
 * call order.  Returns 0 (error set) when no set could be built. */
static int space_device_ready_(cpSpace *sp)
{
	if(sp->dev && (sp->structDirty || space_structure_changed(sp))){
		DevSet *old = sp->dev;
		space_detach(sp);
		cpSpace *one[1] = { sp };
		DevSet *ds = devset_build(one, 1, old);
		if(!ds){
			sp->dev = old; sp->world = 0; sp->structDirty = 1;
			return 0;
		}
		devset_free(old);
		sp->ownsDev = 1;
		if(!sleep_apply_edits_(sp)) return 0;
	}
	if(!sp->dev){
		cpSpace *one[1] = { sp };
		DevSet *ds = devset_build(one, 1, NULL);
		if(!ds) return 0;
		sp->ownsDev = 1;
		if(!sleep_apply_edits_(sp)) return 0;
	}
	return 1;
}

/* Bodies with their own position function (cpSpaceStep.c:362-366).  The
 * functions run on the host before the step, over the awake bodies in
 * order with the space locked; their results (position, angle, transform,
 * bias velocities and velocities) are kept and the bodies put back; the
 * device's part 7 updates every body's position as usual, the kept results
 * replace those bodies' values, and part 8 goes on with the shape caches. */
typedef struct PositionOut { int index; double v[15], orig[15]; } PositionOut;

static inline const cpBody *rd(const cpBody *b);

static int position_callbacks_(cpSpace *sp)
{
	for(int i = 0; i < sp->ndyn; i++) if(sp->dyn[i]->position_func != cpBodyUpdatePosition) return 1;
	return 0;
}

static void body_pos_get_(const cpBody *b, double *o)
{
	o[0] = b->p.x; o[1] = b->p.y; o[2] = b->a;
	o[3] = b->transform.a; o[4] = b->transform.b; o[5] = b->transform.c;
	o[6] = b->transform.d; o[7] = b->transform.tx; o[8] = b->transform.ty;
	o[9] = b->v_bias.x; o[10] = b->v_bias.y; o[11] = b->w_bias;
	o[12] = b->v.x; o[13] = b->v.y; o[14] = b->w;
}

static int run_position_funcs_(cpSpace *sp, cpFloat dt, PositionOut **out)
{
	PositionOut *o = HALLOC(PositionOut, sp->ndyn > 0 ? sp->ndyn : 1);
	int n = 0;
	sp->locked++;
	for(int i = 0; i < sp->ndyn; i++){
		cpBody *b = sp->dyn[i];
		if(b->position_func == cpBodyUpdatePosition) continue;
		rd(b);
		PositionOut *r = &o[n++];
		r->index = i;
		body_pos_get_(b, r->orig);
		b->position_func(b, dt);
		rd(b);
		body_pos_get_(b, r->v);
	}
	space_unlock_(sp);
	/* the bodies as the device holds them until its update */
	for(int k = 0; k < n; k++){
		cpBody *b = sp->dyn[o[k].index];
		const double *q = o[k].orig;
		b->p = cpv(q[0], q[1]); b->a = q[2];
		b->transform = (cpTransform){q[3], q[4], q[5], q[6], q[7], q[8]};
		b->v_bias = cpv(q[9], q[10]); b->w_bias = q[11];
		b->v = cpv(q[12], q[13]); b->w = q[14];
	}
	*out = o;
	return n;
}

static int put_positions_(cpSpace *sp, const PositionOut *o, int n)
{
	DevSet *ds = sp->dev;
	size_t off = (size_t)ds->hworld[sp->world].bodyOff;
	int ok = 1;
	for(int k = 0; k < n && ok; k++){
		size_t g = off + (size_t)o[k].index;
		double *dst[15] = { ds->d.px, ds->d.py, ds->d.ang, ds->d.ta, ds->d.tb, ds->d.tc, ds->d.td, ds->d.ttx, ds->d.tty,
		                    ds->d.vbx, ds->d.vby, ds->d.wb, ds->d.vx, ds->d.vy, ds->d.w };
		for(int j = 0; j < 15; j++) ok &= h2d(dst[j] + g, &o[k].v[j], sizeof(double));
	}
	if(!ok){ set_error(CP_GPU_ERR_CUDA, "position functions: upload failed"); return -1; }
	return 0;
}

/* Bodies with their own velocity function (cpSpaceStep.c:399-403).  The
 * functions run on the host after the joints' pre-solve callbacks, in the
 * order of the awake bodies, with the space locked, on the state the
 * device's velocity update would read (a body with one is not allowed a
 * damped spring, whose pre-step impulse the device adds first); a function
 * that reads another body's velocity sees the bodies with the default
 * update before it, and the earlier ones with their own functions after.  Their
 * results (velocity, angular velocity, the force and torque left behind)
 * are kept and the bodies put back; the device then updates every body as
 * usual (part 5) and the kept results replace the updates of these bodies,
 * packed solver records included, before the solve (part 6). */
typedef struct VelocityOut { int index; double v[6], orig[6]; } VelocityOut;

static int velocity_callbacks_(cpSpace *sp)
{
	for(int i = 0; i < sp->ndyn; i++) if(sp->dyn[i]->velocity_func != cpBodyUpdateVelocity) return 1;
	return 0;
}

static int run_velocity_funcs_(cpSpace *sp, cpFloat dt, VelocityOut **out)
{
	/* the joints' pre-solve edits go up first: the device must read them */
	devset_flush_space(sp->dev, sp->world);
	VelocityOut *o = HALLOC(VelocityOut, sp->ndyn > 0 ? sp->ndyn : 1);
	int n = 0;
	cpVect g = sp->gravity;
	cpFloat damping = pow(sp->damping, dt);
	sp->locked++;
	for(int i = 0; i < sp->ndyn; i++){
		cpBody *b = sp->dyn[i];
		if(b->velocity_func == cpBodyUpdateVelocity) continue;
		rd(b);
		VelocityOut *r = &o[n++];
		r->index = i;
		r->orig[0] = b->v.x; r->orig[1] = b->v.y; r->orig[2] = b->w;
		r->orig[3] = b->f.x; r->orig[4] = b->f.y; r->orig[5] = b->t;
		b->velocity_func(b, g, damping, dt);
		rd(b);
		r->v[0] = b->v.x; r->v[1] = b->v.y; r->v[2] = b->w;
		r->v[3] = b->f.x; r->v[4] = b->f.y; r->v[5] = b->t;
	}
	space_unlock_(sp);
	/* the bodies as the device holds them until its update */
	for(int k = 0; k < n; k++){
		cpBody *b = sp->dyn[o[k].index];
		b->v = cpv(o[k].orig[0], o[k].orig[1]); b->w = o[k].orig[2];
		b->f = cpv(o[k].orig[3], o[k].orig[4]); b->t = o[k].orig[5];
	}
	*out = o;
	return n;
}

static int put_velocities_(cpSpace *sp, const VelocityOut *o, int n)
{
	DevSet *ds = sp->dev;
	size_t off = (size_t)ds->hworld[sp->world].bodyOff;
	int ok = 1;
	for(int k = 0; k < n && ok; k++){
		size_t g = off + (size_t)o[k].index;
		ok &= h2d(ds->d.vx + g, &o[k].v[0], sizeof(double));
		ok &= h2d(ds->d.vy + g, &o[k].v[1], sizeof(double));
		ok &= h2d(ds->d.w + g, &o[k].v[2], sizeof(double));
		ok &= h2d(ds->d.fx + g, &o[k].v[3], sizeof(double));
		ok &= h2d(ds->d.fy + g, &o[k].v[4], sizeof(double));
		ok &= h2d(ds->d.tq + g, &o[k].v[5], sizeof(double));
		ok &= h2d(ds->d.pbody + 8*g, &o[k].v[0], 3*sizeof(double));   /* packed vx, vy, w */
	}
	if(!ok){ set_error(CP_GPU_ERR_CUDA, "velocity functions: upload failed"); return -1; }
	return 0;
}

/* The joints' pre-solve callbacks (cpSpaceStep.c:389-396; run before the
 * device's pre-step, their edits uploaded with it) or post-solve callbacks
 * (:428-434; after the solve, the accumulators read back on demand), over
 * the awake joints in the space's order, with the space locked. */
static int constraint_callbacks_(cpSpace *sp)
{
	for(int i = 0; i < sp->ncons; i++) if(sp->cons[i]->preSolve || sp->cons[i]->postSolve) return 1;
	return 0;
}

static void constraints_solve_callbacks_(cpSpace *sp, int post)
{
	sp->locked++;
	for(int i = 0; i < sp->ncons; i++){
		cpConstraint *c = sp->cons[i];
		if(!post && c->preSolve) c->preSolve(c, sp);
		if(post && c->postSolve) c->postSolve(c, sp);
	}
	space_unlock_(sp);
}

void cpSpaceStep(cpSpace *sp, cpFloat dt)
{
	if(dt == 0.0) return;
	if(!space_supported(sp)) return;
	if(sp->dev && !sp->ownsDev){
		set_error(CP_GPU_ERR_UNSUPPORTED, "space belongs to a cpGpuBatch; step it with cpGpuBatchStep");
		return;
	}
	if(!space_device_ready_(sp)) return;
	double dts[1] = { dt };
	int sleep = sleep_mode_(sp), bridge = sp->handlersOn, jcb = constraint_callbacks_(sp), vcb = velocity_callbacks_(sp);
	int pcb = position_callbacks_(sp);
	if(sleep || bridge || jcb || vcb || pcb){
		/* the host's parts of the step between the device's: the handlers'
		 * begin and pre-solve (cpSpaceStep.c:259-286), cpSpaceProcessComponents
		 * (:375), separate (:307-313), the joints' pre-solve (:389-396) and
		 * post-solve (:428-434), the handlers' post-solve (:439-444) */
		if(sleep) graph_start_(sp); else graph_stop_(sp);
		sp->sleepMutated = 0;
		if(pcb){
			PositionOut *po = NULL;
			int n = run_position_funcs_(sp, dt, &po);
			int rc = devset_step_part(sp->dev, dts, NULL, 7);
			if(rc == 0) rc = put_positions_(sp, po, n);
			free(po);
			if(rc != 0 || devset_step_part(sp->dev, dts, NULL, 8) != 0) return;
		} else if(devset_step_part(sp->dev, dts, NULL, 1) != 0) return;
		if(bridge && !handlers_collide_(sp)) return;
		if(sleep && !sleep_sync_(sp, dt)) return;
		if(bridge || jcb || vcb){
			if(devset_step_part(sp->dev, dts, NULL, 3) != 0) return;
			if(bridge && !handlers_separate_(sp)) return;
			if(jcb) constraints_solve_callbacks_(sp, 0);
			if(vcb){
				VelocityOut *vo = NULL;
				int n = run_velocity_funcs_(sp, dt, &vo);
				int rc = devset_step_part(sp->dev, dts, NULL, 5);
				if(rc == 0) rc = put_velocities_(sp, vo, n);
				free(vo);
				if(rc != 0 || devset_step_part(sp->dev, dts, NULL, 6) != 0) return;
			} else if(devset_step_part(sp->dev, dts, NULL, 4) != 0) return;
			if(jcb) constraints_solve_callbacks_(sp, 1);
			if(bridge && !handlers_post_solve_(sp)) return;
		} else {
			devset_step_part(sp->dev, dts, NULL, 2);
		}
	} else {
		graph_stop_(sp);
		devset_step(sp->dev, dts, NULL);
	}
	run_post_step_(sp);
}

static inline const cpBody *rd(const cpBody *b);

/* Every dynamic body's public state in one read: 8 doubles per body in
 * the space's body order (position, velocity, angle, angular velocity,
 * rotation), the values the getters return.  After a step they are
 * gathered on the device and copied in one transfer. */
int cpGpuSpaceGetBodyStates(cpSpace *sp, double *out, int max)
{
	if(!sp || (max > 0 && !out)){ set_error(CP_GPU_ERR_ARGUMENT, "body states: null argument"); return -1; }
	int n = sp->ndyn < max ? sp->ndyn : max;
	if(n <= 0) return 0;
	if(!sp->dev || sp->bodyDirty || sp->structDirty || !sp->hostStale){
		/* the host structs hold the current state */
		for(int i = 0; i < n; i++){
			const cpBody *b = rd(sp->dyn[i]);
			double *o = out + 8*(size_t)i;
			cpVect p = cpTransformPoint(b->transform, cpvzero);
			o[0] = p.x; o[1] = p.y; o[2] = b->v.x; o[3] = b->v.y;
			o[4] = b->a; o[5] = b->w; o[6] = b->transform.a; o[7] = b->transform.b;
		}
		return n;
	}
	DevSet *ds = sp->dev;
	if(ds->bstatesCap < n){
		if(ds->bstates) cudaFree(ds->bstates);
		ds->bstates = NULL; ds->bstatesCap = 0;
		if(!cuda_ok(cudaMalloc((void **)&ds->bstates, sizeof(double)*8*(size_t)n), "cudaMalloc body states")) return -1;
		ds->bstatesCap = n;
	}
	cudaStream_t st = lib_stream();
	if(cpg_launch_body_states(&ds->d, sp->world, ds->bstates, n, st) != 0){ set_error(CP_GPU_ERR_CUDA, "body states launch failed"); return -1; }
	if(!d2h(out, ds->bstates, sizeof(double)*8*(size_t)n) || !cuda_ok(cudaStreamSynchronize(st), "body states")) return -1;
	check_stats(ds);
	return n;
}

/* ====================================================================
 * Saved states of a space: a device copy of its whole set (bodies, shape
 * caches, the trees and pair caches, the arbiter table and contacts,
 * joints with their accumulated impulses) and the host counters that go
 * with it (timestamp, last dt, the dt the joint bias terms were made for).
 * The same copy is what the differentiable rollout keeps per segment.
 * ==================================================================== */
struct cpGpuSpaceState {
	cpSpace *space;
	DevSet *ds;
	unsigned long long editGen;
	void *slab;
	size_t bytes;
	cpTimestamp stamp;
	cpFloat currDt, jointDt;
};

cpGpuSpaceState *cpGpuSpaceSaveState(cpSpace *sp)
{
	if(!sp){ set_error(CP_GPU_ERR_ARGUMENT, "save state: null space"); return NULL; }
	if(sp->dev && !sp->ownsDev){ set_error(CP_GPU_ERR_UNSUPPORTED, "save state: the space belongs to a cpGpuBatch"); return NULL; }
	if(sleep_mode_(sp)){ set_error(CP_GPU_ERR_UNSUPPORTED, "save state: sleeping keeps host state that is not saved"); return NULL; }
	if(!space_device_ready_(sp)) return NULL;
	DevSet *ds = sp->dev;
	devset_flush_space(ds, sp->world);
	check_stats(ds);
	cpGpuSpaceState *st = (cpGpuSpaceState *)calloc(1, sizeof(cpGpuSpaceState));
	if(!st) return NULL;
	if(!cuda_ok(cudaMalloc(&st->slab, ds->slabBytes), "cudaMalloc saved state")){ free(st); return NULL; }
	st->bytes = ds->slabBytes;
	if(!cuda_ok(cudaMemcpyAsync(st->slab, ds->slab, ds->slabBytes, cudaMemcpyDeviceToDevice, lib_stream()), "save state") ||
	   !cuda_ok(cudaStreamSynchronize(lib_stream()), "save state")){
		cudaFree(st->slab); free(st); return NULL;
	}
	st->space = sp; st->ds = ds; st->editGen = sp->editGen;
	st->stamp = sp->stamp; st->currDt = sp->curr_dt; st->jointDt = sp->jointDt;
	return st;
}

int cpGpuSpaceRestoreState(cpSpace *sp, const cpGpuSpaceState *st)
{
	if(!sp || !st){ set_error(CP_GPU_ERR_ARGUMENT, "restore state: null argument"); return CP_GPU_ERR_ARGUMENT; }
	if(st->space != sp || sp->dev != st->ds || sp->structDirty || space_structure_changed(sp) || st->bytes != sp->dev->slabBytes){
		set_error(CP_GPU_ERR_UNSUPPORTED, "restore state: the space's objects were added or removed since the save");
		return CP_GPU_ERR_UNSUPPORTED;
	}
	if(sp->editGen != st->editGen){
		set_error(CP_GPU_ERR_UNSUPPORTED, "restore state: objects of the space were edited since the save");
		return CP_GPU_ERR_UNSUPPORTED;
	}
	DevSet *ds = sp->dev;
	check_stats(ds);
	if(!cuda_ok(cudaMemcpyAsync(ds->slab, st->slab, st->bytes, cudaMemcpyDeviceToDevice, lib_stream()), "restore state") ||
	   !cuda_ok(cudaStreamSynchronize(lib_stream()), "restore state"))
		return CP_GPU_ERR_CUDA;
	sp->stamp = st->stamp; sp->curr_dt = st->currDt; sp->jointDt = st->jointDt;
	sp->hostStale = 1; sp->consStale = 1; sp->shapesStale = 1; sp->snapValid = 0;
	return CP_GPU_OK;
}

void cpGpuSpaceStateFree(cpGpuSpaceState *st)
{
	if(!st) return;
	if(st->slab) cudaFree(st->slab);
	free(st);
}

/* ====================================================================
 * Spatial queries (cpSpaceQuery.c:48-204, cpShape.c:222-256): answered on
 * the device by cpg_query.cu, which walks the space's trees in the
 * reference's order; the callbacks then run here, in that order.
 * ==================================================================== */
#define CPG_QUERY_HITS0 64

static cpgQuery query_new_(int kind, double ax, double ay, double bx, double by, double r, cpShapeFilter f)
{
	cpgQuery q;
	memset(&q, 0, sizeof(q));
	q.kind = kind; q.ax = ax; q.ay = ay; q.bx = bx; q.by = by; q.r = r;
	q.group = (unsigned long long)f.group; q.cat = f.categories; q.mask = f.mask;
	return q;
}

/* Runs nq queries on the space's device set.  On success *hits holds cap
 * records per query and *counts the number of each (all-hits queries) or
 * 0/1 (nearest and first-hit queries); both are malloc'd. */
static int run_queries_(cpSpace *sp, const cpgQuery *q, int nq, cpgHit **hitsOut, int **countsOut, int *capOut)
{
	*hitsOut = NULL; *countsOut = NULL; *capOut = 0;
	if(!sp || nq < 0 || (nq > 0 && !q)){ set_error(CP_GPU_ERR_ARGUMENT, "query: null space or queries"); return 0; }
	if(sp->dev && !sp->ownsDev){
		if(sp->structDirty || space_structure_changed(sp)){
			set_error(CP_GPU_ERR_UNSUPPORTED, "query: objects were added to or removed from a space of a cpGpuBatch");
			return 0;
		}
	} else if(!space_device_ready_(sp)) return 0;
	DevSet *ds = sp->dev;
	devset_flush_space(ds, sp->world);
	cudaStream_t st = lib_stream();
	int brute = (sp->mode == CP_GPU_SOLVER_COLORED);
	int cap = CPG_QUERY_HITS0;
	int *counts = HALLOC(int, nq + 1);
	for(int attempt = 0; attempt < 2; attempt++){
		size_t qb = align256(sizeof(cpgQuery)*(size_t)(nq > 0 ? nq : 1));
		size_t hb = align256(sizeof(cpgHit)*(size_t)(nq > 0 ? nq : 1)*(size_t)cap);
		size_t cb = align256(sizeof(int)*(size_t)(nq + 1));
		size_t need = qb + hb + cb;
		if(ds->qbytes < need){
			if(ds->qbuf) cudaFree(ds->qbuf);
			ds->qbuf = NULL; ds->qbytes = 0;
			if(!cuda_ok(cudaMalloc(&ds->qbuf, need), "cudaMalloc queries")){ free(counts); return 0; }
			ds->qbytes = need;
		}
		char *base = (char *)ds->qbuf;
		cpgQuery *dq = (cpgQuery *)base;
		cpgHit *dh = (cpgHit *)(base + qb);
		int *dc = (int *)(base + qb + hb);
		int ok = h2d(dq, q, sizeof(cpgQuery)*(size_t)nq);
		ok &= cuda_ok(cudaMemsetAsync(dc + nq, 0, sizeof(int), st), "query status");
		ok &= (cpg_launch_query(&ds->d, sp->world, dq, nq, dh, cap, dc, brute, dc + nq, st) == 0);
		ok &= d2h(counts, dc, sizeof(int)*(size_t)(nq + 1));
		ok &= cuda_ok(cudaStreamSynchronize(st), "query");
		if(!ok){ set_error(CP_GPU_ERR_CUDA, "query launch failed"); free(counts); return 0; }
		if(counts[nq]){
			set_error(CP_GPU_ERR_OVERFLOW, "query: tree walk stack or guard exceeded");
			free(counts); return 0;
		}
		int most = 0;
		for(int i = 0; i < nq; i++) if(counts[i] > most) most = counts[i];
		if(most > cap && attempt == 0){ cap = most; continue; }
		cpgHit *hits = HALLOC(cpgHit, (size_t)(nq > 0 ? nq : 1)*(size_t)cap);
		if(!d2h(hits, dh, sizeof(cpgHit)*(size_t)nq*(size_t)cap) || !cuda_ok(cudaStreamSynchronize(st), "query results")){
			free(hits); free(counts); return 0;
		}
		*hitsOut = hits; *countsOut = counts; *capOut = cap;
		return 1;
	}
	set_error(CP_GPU_ERR_OVERFLOW, "query: hit lists kept growing");
	free(counts);
	return 0;
}

static cpShape *slot_shape_(cpSpace *sp, int slot)
{
	return (slot >= 0 && slot < sp->nshapes) ? sp->shapes[slot] : NULL;
}

void cpSpacePointQuery(cpSpace *sp, cpVect point, cpFloat maxDistance, cpShapeFilter filter, cpSpacePointQueryFunc func, void *data)
{
	cpgQuery q = query_new_(CPG_Q_POINT, point.x, point.y, 0.0, 0.0, maxDistance, filter);
	cpgHit *h; int *c, cap;
	if(!run_queries_(sp, &q, 1, &h, &c, &cap)) return;
	sp->locked++;
	for(int k = 0; k < c[0] && k < cap; k++){
		cpShape *shape = slot_shape_(sp, h[k].shape);
		if(shape && func) func(shape, cpv(h[k].px, h[k].py), h[k].d, cpv(h[k].gx, h[k].gy), data);
	}
	free(h); free(c);
	space_unlock_(sp);
	run_post_step_(sp);
}

cpShape *cpSpacePointQueryNearest(cpSpace *sp, cpVect point, cpFloat maxDistance, cpShapeFilter filter, cpPointQueryInfo *out)
{
	cpPointQueryInfo info = {NULL, cpvzero, maxDistance, cpvzero};
	if(out) *out = info; else out = &info;
	cpgQuery q = query_new_(CPG_Q_POINT_NEAREST, point.x, point.y, 0.0, 0.0, maxDistance, filter);
	cpgHit *h; int *c, cap;
	if(!run_queries_(sp, &q, 1, &h, &c, &cap)) return NULL;
	if(c[0] && slot_shape_(sp, h[0].shape)){
		out->shape = slot_shape_(sp, h[0].shape);
		out->point = cpv(h[0].px, h[0].py);
		out->distance = h[0].d;
		out->gradient = cpv(h[0].gx, h[0].gy);
	}
	free(h); free(c);
	return (cpShape *)out->shape;
}

void cpSpaceSegmentQuery(cpSpace *sp, cpVect start, cpVect end, cpFloat radius, cpShapeFilter filter, cpSpaceSegmentQueryFunc func, void *data)
{
	cpgQuery q = query_new_(CPG_Q_SEGMENT, start.x, start.y, end.x, end.y, radius, filter);
	cpgHit *h; int *c, cap;
	if(!run_queries_(sp, &q, 1, &h, &c, &cap)) return;
	sp->locked++;
	for(int k = 0; k < c[0] && k < cap; k++){
		cpShape *shape = slot_shape_(sp, h[k].shape);
		if(shape && func) func(shape, cpv(h[k].px, h[k].py), cpv(h[k].gx, h[k].gy), h[k].d, data);
	}
	free(h); free(c);
	space_unlock_(sp);
	run_post_step_(sp);
}

cpShape *cpSpaceSegmentQueryFirst(cpSpace *sp, cpVect start, cpVect end, cpFloat radius, cpShapeFilter filter, cpSegmentQueryInfo *out)
{
	cpSegmentQueryInfo info = {NULL, end, cpvzero, 1.0};
	if(out) *out = info; else out = &info;
	cpgQuery q = query_new_(CPG_Q_SEGMENT_FIRST, start.x, start.y, end.x, end.y, radius, filter);
	cpgHit *h; int *c, cap;
	if(!run_queries_(sp, &q, 1, &h, &c, &cap)) return NULL;
	if(c[0] && slot_shape_(sp, h[0].shape)){
		out->shape = slot_shape_(sp, h[0].shape);
		out->point = cpv(h[0].px, h[0].py);
		out->normal = cpv(h[0].gx, h[0].gy);
		out->alpha = h[0].d;
	}
	free(h); free(c);
	return (cpShape *)out->shape;
}

void cpSpaceBBQuery(cpSpace *sp, cpBB bb, cpShapeFilter filter, cpSpaceBBQueryFunc func, void *data)
{
	cpgQuery q = query_new_(CPG_Q_BB, bb.l, bb.b, bb.r, bb.t, 0.0, filter);
	cpgHit *h; int *c, cap;
	if(!run_queries_(sp, &q, 1, &h, &c, &cap)) return;
	sp->locked++;
	for(int k = 0; k < c[0] && k < cap; k++){
		cpShape *shape = slot_shape_(sp, h[k].shape);
		if(shape && func) func(shape, data);
	}
	free(h); free(c);
	space_unlock_(sp);
	run_post_step_(sp);
}

/* The slot of a shape in its space, or -1 (error set) when it is in none. */
static int shape_slot_(const cpShape *shape)
{
	cpSpace *sp = shape ? shape->space : NULL;
	if(!sp){
		set_error(CP_GPU_ERR_UNSUPPORTED, "shape query: the shape is in no space (its geometry lives on the device)");
		return -1;
	}
	for(int i = 0; i < sp->nshapes; i++) if(sp->shapes[i] == shape) return i;
	set_error(CP_GPU_ERR_ARGUMENT, "shape query: shape not found in its space");
	return -1;
}

cpFloat cpShapePointQuery(const cpShape *shape, cpVect p, cpPointQueryInfo *out)
{
	cpPointQueryInfo blank = {NULL, cpvzero, INFINITY, cpvzero};
	if(out) *out = blank; else out = &blank;
	int slot = shape_slot_(shape);
	if(slot < 0) return out->distance;
	cpgQuery q = query_new_(CPG_Q_SHAPE_POINT, p.x, p.y, 0.0, 0.0, 0.0, CP_SHAPE_FILTER_ALL);
	q.pad = slot;
	cpgHit *h; int *c, cap;
	if(!run_queries_(shape->space, &q, 1, &h, &c, &cap)) return out->distance;
	if(c[0]){
		out->shape = shape;
		out->point = cpv(h[0].px, h[0].py);
		out->distance = h[0].d;
		out->gradient = cpv(h[0].gx, h[0].gy);
	}
	free(h); free(c);
	return out->distance;
}

cpBool cpShapeSegmentQuery(const cpShape *shape, cpVect a, cpVect b, cpFloat radius, cpSegmentQueryInfo *info)
{
	cpSegmentQueryInfo blank = {NULL, b, cpvzero, 1.0};
	if(info) *info = blank; else info = &blank;
	int slot = shape_slot_(shape);
	if(slot < 0) return cpFalse;
	cpgQuery q = query_new_(CPG_Q_SHAPE_SEGMENT, a.x, a.y, b.x, b.y, radius, CP_SHAPE_FILTER_ALL);
	q.pad = slot;
	cpgHit *h; int *c, cap;
	if(!run_queries_(shape->space, &q, 1, &h, &c, &cap)) return cpFalse;
	if(c[0]){
		info->shape = shape;
		info->point = cpv(h[0].px, h[0].py);
		info->normal = cpv(h[0].gx, h[0].gy);
		info->alpha = h[0].d;
	}
	free(h); free(c);
	return info->shape != NULL;
}

static cpBB shape_cache_(cpShape *s, cpTransform t);
static void shapes_pull_all_(cpSpace *sp);

/* A shape's host cache as a probe; its polygon planes go to planes (four
 * arrays of n) from voff on. */
static void probe_fill_(const cpShape *s, cpgProbe *p, double *planes, int n, int voff)
{
	memset(p, 0, sizeof(*p));
	p->kind = s->kind; p->r = s->r;
	cpVect g0 = (s->kind == CPG_CIRCLE) ? s->tc : s->ta;
	p->p0x = g0.x; p->p0y = g0.y; p->p1x = s->tb.x; p->p1y = s->tb.y; p->nx = s->tn.x; p->ny = s->tn.y;
	p->atx = s->a_tangent.x; p->aty = s->a_tangent.y; p->btx = s->b_tangent.x; p->bty = s->b_tangent.y;
	p->rotx = s->body ? s->body->transform.a : 1.0;
	p->roty = s->body ? s->body->transform.b : 0.0;
	p->bbl = s->bb.l; p->bbb = s->bb.b; p->bbr = s->bb.r; p->bbt = s->bb.t;
	p->hashid = (unsigned long long)s->hashid;
	p->group = (unsigned long long)s->filter.group; p->cat = s->filter.categories; p->mask = s->filter.mask;
	p->sensor = s->sensor ? 1 : 0;
	p->count = (s->kind == CPG_POLY) ? s->count : 0;
	p->voff = voff;
	p->slot = -1;
	for(int i = 0; i < p->count; i++){
		planes[voff + i] = s->gv[i].x; planes[n + voff + i] = s->gv[i].y;
		planes[2*n + voff + i] = s->gn[i].x; planes[3*n + voff + i] = s->gn[i].y;
	}
}

static cpContactPointSet point_set_(const cpgShapeHit *h)
{
	cpContactPointSet set;
	memset(&set, 0, sizeof(set));
	set.count = h->count;
	set.normal = cpv(h->nx, h->ny);
	for(int i = 0; i < h->count && i < CP_MAX_CONTACTS_PER_ARBITER; i++){
		set.points[i].pointA = cpv(h->ax[i], h->ay[i]);
		set.points[i].pointB = cpv(h->bx[i], h->by[i]);
		set.points[i].distance = h->dist[i];
	}
	return set;
}

/* cpSpaceQuery.c:230-246: the shape's cache is brought to its body's
 * transform here, as cpShapeUpdate does there; the device walks the trees
 * with it. */
cpBool cpSpaceShapeQuery(cpSpace *sp, cpShape *shape, cpSpaceShapeQueryFunc func, void *data)
{
	if(!sp || !shape){ set_error(CP_GPU_ERR_ARGUMENT, "shape query: null argument"); return cpFalse; }
	if(shape->body){
		rd(shape->body);
		shape_cache_(shape, shape->body->transform);
	} else if(shape->space){
		shapes_pull_all_(shape->space);
	}
	if(sp->dev && !sp->ownsDev){
		if(sp->structDirty || space_structure_changed(sp)){
			set_error(CP_GPU_ERR_UNSUPPORTED, "query: objects were added to or removed from a space of a cpGpuBatch");
			return cpFalse;
		}
	} else if(!space_device_ready_(sp)) return cpFalse;
	DevSet *ds = sp->dev;
	devset_flush_space(ds, sp->world);
	cudaStream_t st = lib_stream();
	int nplanes = (shape->kind == CPG_POLY) ? shape->count : 0;
	double *hplanes = HALLOC(double, 4*(size_t)(nplanes > 0 ? nplanes : 1));
	cpgProbe probe;
	probe_fill_(shape, &probe, hplanes, nplanes, 0);
	if(shape->space == sp) for(int i = 0; i < sp->nshapes; i++) if(sp->shapes[i] == shape){ probe.slot = i; break; }
	int brute = (sp->mode == CP_GPU_SOLVER_COLORED);
	int cap = CPG_QUERY_HITS0, counts[3] = {0, 0, 0};
	cpgShapeHit *hits = NULL;
	cpBool any = cpFalse;
	for(int attempt = 0; attempt < 2; attempt++){
		size_t pb = align256(sizeof(double)*4*(size_t)(nplanes > 0 ? nplanes : 1));
		size_t hb = align256(sizeof(cpgShapeHit)*(size_t)cap);
		size_t need = pb + hb + 256;
		if(ds->qbytes < need){
			if(ds->qbuf) cudaFree(ds->qbuf);
			ds->qbuf = NULL; ds->qbytes = 0;
			if(!cuda_ok(cudaMalloc(&ds->qbuf, need), "cudaMalloc queries")){ free(hplanes); return cpFalse; }
			ds->qbytes = need;
		}
		char *base = (char *)ds->qbuf;
		double *dplanes = (double *)base;
		cpgShapeHit *dh = (cpgShapeHit *)(base + pb);
		int *dc = (int *)(base + pb + hb);
		int ok = h2d(dplanes, hplanes, sizeof(double)*4*(size_t)nplanes);
		ok &= (cpg_launch_shape_query(&ds->d, sp->world, &probe, dplanes, nplanes, brute, dh, cap, dc, st) == 0);
		ok &= d2h(counts, dc, sizeof(int)*3);
		ok &= cuda_ok(cudaStreamSynchronize(st), "shape query");
		if(!ok){ set_error(CP_GPU_ERR_CUDA, "shape query launch failed"); free(hplanes); return cpFalse; }
		if(counts[2]){ set_error(CP_GPU_ERR_OVERFLOW, "shape query: tree walk stack or guard exceeded"); free(hplanes); return cpFalse; }
		if(counts[0] > cap && attempt == 0){ cap = counts[0]; continue; }
		hits = HALLOC(cpgShapeHit, cap);
		if(!d2h(hits, dh, sizeof(cpgShapeHit)*(size_t)cap) || !cuda_ok(cudaStreamSynchronize(st), "shape query results")){
			free(hits); free(hplanes); return cpFalse;
		}
		break;
	}
	free(hplanes);
	if(!hits) return cpFalse;
	int n = counts[0] < cap ? counts[0] : cap;
	sp->locked++;
	for(int k = 0; k < n; k++){
		cpShape *other = slot_shape_(sp, hits[k].shape);
		if(!other) continue;
		cpContactPointSet set = point_set_(&hits[k]);
		if(func) func(other, &set, data);
	}
	space_unlock_(sp);
	any = counts[1] ? cpTrue : cpFalse;
	free(hits);
	run_post_step_(sp);
	return any;
}

/* cpShape.c:258-283 on the shapes' caches as they are */
cpContactPointSet cpShapesCollide(const cpShape *a, const cpShape *b)
{
	cpContactPointSet set;
	memset(&set, 0, sizeof(set));
	if(!a || !b){ set_error(CP_GPU_ERR_ARGUMENT, "cpShapesCollide: null shape"); return set; }
	if(!device_available()) return set;
	if(a->space) shapes_pull_all_(a->space);
	if(b->space && b->space != a->space) shapes_pull_all_(b->space);
	static void *buf = NULL;
	static size_t bufBytes = 0;
	int na = (a->kind == CPG_POLY) ? a->count : 0, nb = (b->kind == CPG_POLY) ? b->count : 0;
	int n = na + nb;
	double *hplanes = HALLOC(double, 4*(size_t)(n > 0 ? n : 1));
	cpgProbe probes[2];
	probe_fill_(a, &probes[0], hplanes, n, 0);
	probe_fill_(b, &probes[1], hplanes, n, na);
	size_t pb = align256(sizeof(cpgProbe)*2), lb = align256(sizeof(double)*4*(size_t)(n > 0 ? n : 1));
	size_t need = pb + lb + align256(sizeof(cpgShapeHit)) + 256;
	if(bufBytes < need){
		if(buf) cudaFree(buf);
		buf = NULL; bufBytes = 0;
		if(!cuda_ok(cudaMalloc(&buf, need), "cudaMalloc cpShapesCollide")){ free(hplanes); return set; }
		bufBytes = need;
	}
	char *base = (char *)buf;
	cpgProbe *dp = (cpgProbe *)base;
	double *dl = (double *)(base + pb);
	cpgShapeHit *dh = (cpgShapeHit *)(base + pb + lb);
	int *dc = (int *)(base + pb + lb + align256(sizeof(cpgShapeHit)));
	cudaStream_t st = lib_stream();
	cpgShapeHit h;
	int cnt = 0;
	int ok = h2d(dp, probes, sizeof(probes)) && h2d(dl, hplanes, sizeof(double)*4*(size_t)n);
	ok = ok && cpg_launch_shape_pair(dp, dl, n, dh, dc, st) == 0;
	ok = ok && d2h(&h, dh, sizeof(h)) && d2h(&cnt, dc, sizeof(int)) && cuda_ok(cudaStreamSynchronize(st), "cpShapesCollide");
	free(hplanes);
	if(!ok){ set_error(CP_GPU_ERR_CUDA, "cpShapesCollide launch failed"); return set; }
	return point_set_(&h);
}

/* Many nearest-point or first-hit queries in one launch, one thread each. */
int cpGpuSpacePointQueryNearestBatch(cpSpace *sp, int n, const cpVect *points, cpFloat maxDistance,
                                     cpShapeFilter filter, cpPointQueryInfo *out)
{
	if(n < 0 || (n > 0 && (!points || !out))){ set_error(CP_GPU_ERR_ARGUMENT, "query batch: bad arguments"); return CP_GPU_ERR_ARGUMENT; }
	cpgQuery *q = HALLOC(cpgQuery, n);
	for(int i = 0; i < n; i++) q[i] = query_new_(CPG_Q_POINT_NEAREST, points[i].x, points[i].y, 0.0, 0.0, maxDistance, filter);
	cpgHit *h; int *c, cap;
	if(!run_queries_(sp, q, n, &h, &c, &cap)){ free(q); return g_error ? g_error : CP_GPU_ERR_CUDA; }
	for(int i = 0; i < n; i++){
		cpPointQueryInfo info = {NULL, cpvzero, maxDistance, cpvzero};
		const cpgHit *r = h + (size_t)i*cap;
		if(c[i] && slot_shape_(sp, r->shape)){
			info.shape = slot_shape_(sp, r->shape);
			info.point = cpv(r->px, r->py); info.distance = r->d; info.gradient = cpv(r->gx, r->gy);
		}
		out[i] = info;
	}
	free(h); free(c); free(q);
	return CP_GPU_OK;
}

int cpGpuSpaceSegmentQueryFirstBatch(cpSpace *sp, int n, const cpVect *starts, const cpVect *ends, cpFloat radius,
                                     cpShapeFilter filter, cpSegmentQueryInfo *out)
{
	if(n < 0 || (n > 0 && (!starts || !ends || !out))){ set_error(CP_GPU_ERR_ARGUMENT, "query batch: bad arguments"); return CP_GPU_ERR_ARGUMENT; }
	cpgQuery *q = HALLOC(cpgQuery, n);
	for(int i = 0; i < n; i++) q[i] = query_new_(CPG_Q_SEGMENT_FIRST, starts[i].x, starts[i].y, ends[i].x, ends[i].y, radius, filter);
	cpgHit *h; int *c, cap;
	if(!run_queries_(sp, q, n, &h, &c, &cap)){ free(q); return g_error ? g_error : CP_GPU_ERR_CUDA; }
	for(int i = 0; i < n; i++){
		cpSegmentQueryInfo info = {NULL, ends[i], cpvzero, 1.0};
		const cpgHit *r = h + (size_t)i*cap;
		if(c[i] && slot_shape_(sp, r->shape)){
			info.shape = slot_shape_(sp, r->shape);
			info.point = cpv(r->px, r->py); info.normal = cpv(r->gx, r->gy); info.alpha = r->d;
		}
		out[i] = info;
	}
	free(h); free(c); free(q);
	return CP_GPU_OK;
}

void cpGpuSpaceSync(cpSpace *sp)
{
	if(sp && sp->dev){
		cuda_ok(cudaStreamSynchronize(lib_stream()), "sync");
		check_stats(sp->dev);
	}
}

/* ====================================================================
 * Batches
 * ==================================================================== */
/* A differentiable rollout of a batch: the forward's checkpoints. */
/* The light tape of one segment (a cpgTape whose app is NULL): recorded
 * by the forward and kept for the reverse pass. */
typedef struct SegTape {
	cpgTape t;
	void *block;
	size_t bytes;
	int recorded;                 /* holds the forward's steps of the segment */
	int maxStepRows;              /* the most rows of one of its steps */
	int rowsUsed;                 /* rows of all its steps */
} SegTape;

/* Scratch of the reverse pass, shared by the segments: the adjoint state,
 * the per-step contact scratch, the recomputed solves' rows and bodies and
 * their per-iteration records. */
typedef struct AdjMem {
	cpgAdj a;
	double *app;                  /* [segRows][iters][2] AdjApp */
	void *block;
	size_t bytes, segRows, stepRows;
	int K, iters;
} AdjMem;

/* A differentiable rollout of a batch: the forward's checkpoints and light
 * tapes, and the reverse pass's scratch, kept for the next rollout of the
 * same shape (a training loop calls forward and backward repeatedly). */
typedef struct Rollout {
	int steps, K, nckpt;
	double dt;
	char *ckpt;                   /* ckptCap copies of the device set */
	int ckptCap;
	unsigned *stamps;             /* [nckpt][nspaces] host stamps at the checkpoints */
	double *currDt;               /* [nckpt][nspaces] */
	SegTape *segs;                /* [segCap] */
	int segCap;
	size_t rowEst;                /* rows to provide for a segment: the largest need seen */
	char *fin;                    /* the forward's final state during the reverse pass */
	AdjMem adj;
	float replayMs, adjointMs;    /* device time of the last reverse pass (with cpGpuSetTiming(1)) */
} Rollout;

struct cpGpuBatch {
	cpSpace **spaces;
	int n, cap;
	DevSet *dev;
	Rollout *roll;
};

static void rollout_free(Rollout *r)
{
	if(!r) return;
	if(r->ckpt) cudaFree(r->ckpt);
	if(r->fin) cudaFree(r->fin);
	for(int i = 0; i < r->segCap; i++) if(r->segs[i].block) cudaFree(r->segs[i].block);
	if(r->adj.block) cudaFree(r->adj.block);
	free(r->segs);
	free(r->stamps); free(r->currDt);
	free(r);
}

cpGpuBatch *cpGpuBatchNew(void) { return (cpGpuBatch *)calloc(1, sizeof(cpGpuBatch)); }

void cpGpuBatchFree(cpGpuBatch *b)
{
	if(!b) return;
	rollout_free(b->roll);
	if(b->dev){
		for(int i = 0; i < b->n; i++) space_pull(b->spaces[i]);
		devset_free(b->dev);
	}
	free(b->spaces);
	free(b);
}

int cpGpuBatchAddSpace(cpGpuBatch *b, cpSpace *sp)
{
	if(!b || !sp || b->dev || sp->dev){
		set_error(CP_GPU_ERR_ARGUMENT, "spaces join a batch before it is first stepped, and only once");
		return -1;
	}
	push_((void ***)&b->spaces, &b->n, &b->cap, sp);
	return b->n - 1;
}

int cpGpuBatchGetTuning(cpGpuBatch *b, int *out)
{
	if(!b || !b->dev || !out) return 0;
	DevSet *ds = b->dev;
	out[0] = ds->tuneBest >= 0 ? tune_threads[ds->tuneBest] : 0;
	out[1] = ds->tuneBest >= 0 ? tune_tree[ds->tuneBest] : -1;
	return 2;
}

int cpGpuBatchStep(cpGpuBatch *b, cpFloat dt, int steps, int use_graph)
{
	if(!b || b->n <= 0) return -1;
	for(int i = 0; i < b->n; i++){
		if(!space_supported(b->spaces[i])) return -1;
		if(sleep_mode_(b->spaces[i])){ set_error(CP_GPU_ERR_UNSUPPORTED, "sleeping runs in a standalone space, not in a cpGpuBatch"); return -1; }
		if(b->spaces[i]->useHash || b->spaces[i]->handlersOn){ set_error(CP_GPU_ERR_UNSUPPORTED, "the spatial hash and collision handlers run in a standalone space, not in a cpGpuBatch"); return -1; }
	}
	if(!b->dev){
		b->dev = devset_build(b->spaces, b->n, NULL);
		if(!b->dev) return -1;
		for(int i = 0; i < b->n; i++) b->spaces[i]->ownsDev = 0;
	}
	double *dts = (double *)malloc(sizeof(double)*(size_t)b->n);
	for(int i = 0; i < b->n; i++) dts[i] = dt;
	int rc = 0;
	b->dev->useGraph = use_graph ? 1 : 0;
	for(int s = 0; s < steps && rc == 0; s++) rc = devset_step(b->dev, dts, NULL);
	b->dev->useGraph = 0;
	free(dts);
	return rc;
}

/* ====================================================================
 * Differentiable rollout (reference-order mode)
 * ==================================================================== */

static int batch_ready(cpGpuBatch *b)
{
	if(!b || b->n == 0){ set_error(CP_GPU_ERR_ARGUMENT, "empty batch"); return 0; }
	for(int i = 0; i < b->n; i++){
		if(!space_supported(b->spaces[i])) return 0;
		if(sleep_mode_(b->spaces[i])){ set_error(CP_GPU_ERR_UNSUPPORTED, "the differentiable rollout does not run sleeping"); return 0; }
		if(b->spaces[i]->mode != CP_GPU_SOLVER_ORDERED){
			set_error(CP_GPU_ERR_UNSUPPORTED, "the differentiable rollout runs the reference-order solver");
			return 0;
		}
	}
	if(!b->dev){
		b->dev = devset_build(b->spaces, b->n, NULL);
		if(!b->dev) return 0;
		for(int i = 0; i < b->n; i++) b->spaces[i]->ownsDev = 0;
	}
	return 1;
}

static void rollout_save(cpGpuBatch *b, int i)
{
	DevSet *ds = b->dev;
	Rollout *r = b->roll;
	for(int w = 0; w < ds->nspaces; w++) devset_flush_space(ds, w);
	cuda_ok(cudaMemcpyAsync(r->ckpt + (size_t)i*ds->slabBytes, ds->slab, ds->slabBytes, cudaMemcpyDeviceToDevice, lib_stream()), "checkpoint");
	for(int w = 0; w < ds->nspaces; w++){
		r->stamps[(size_t)i*ds->nspaces + w] = ds->spaces[w]->stamp;
		r->currDt[(size_t)i*ds->nspaces + w] = ds->spaces[w]->curr_dt;
	}
}

static void rollout_restore_from(DevSet *ds, const char *src, const unsigned *stamps, const double *currDt)
{
	cuda_ok(cudaMemcpyAsync(ds->slab, src, ds->slabBytes, cudaMemcpyDeviceToDevice, lib_stream()), "restore");
	for(int w = 0; w < ds->nspaces; w++){
		cpSpace *sp = ds->spaces[w];
		sp->stamp = stamps[w];
		sp->curr_dt = currDt[w];
		sp->hostStale = 1; sp->consStale = 1; sp->shapesStale = 1; sp->snapValid = 0;
	}
}


/* ---- rollout memory ---- */

#define RCARVE(ptr, type, count) do { size_t b_ = align256(sizeof(type)*(size_t)((count) > 0 ? (count) : 1)); if(base) ptr = (type *)(base + total); total += b_; } while(0)

static size_t seg_carve(const cpgSet *d, cpgTape *t, char *base, int K, size_t rowCap)
{
	size_t total = 0;
	int W = d->nworlds;
	size_t levCap = rowCap + (size_t)K*(W + 1);
	RCARVE(t->body, double, (size_t)K*8*d->totalBodies);
	RCARVE(t->vel, double, (size_t)K*3*d->totalBodies);
	RCARVE(t->shape, double, (size_t)K*6*d->totalShapes);
	RCARVE(t->verts, double, (size_t)K*4*d->totalVerts);
	RCARVE(t->params, cpgParams, (size_t)K*W);
	RCARVE(t->rows, cpgRow, rowCap);
	RCARVE(t->rowInfo, int, 4*rowCap);
	RCARVE(t->rowWorld, int, rowCap);
	RCARVE(t->rowOff, int, (size_t)K*(W + 1));
	RCARVE(t->levels, int, levCap);
	RCARVE(t->levOff, int, (size_t)K*(W + 1));
	RCARVE(t->cursor, int, 4);
	if(base){ t->K = K; t->rowCap = (int)rowCap; t->levCap = (int)levCap; t->app = NULL; t->on = 0; t->step = 0; }
	return total;
}

static size_t adj_carve(const cpgSet *d, AdjMem *m, char *base, int K, size_t segRows, size_t stepRows, int iters)
{
	size_t total = 0;
	size_t nb = (size_t)d->totalBodies, ns = (size_t)d->totalShapes;
	RCARVE(m->a.body, double, 9*nb);
	RCARVE(m->a.arb, double, 4*(size_t)d->arbCap);
	RCARVE(m->a.gMinv, double, nb);
	RCARVE(m->a.gE, double, ns);
	RCARVE(m->a.gU, double, ns);
	RCARVE(m->a.con, double, stepRows*2*4*CPG_ADJ_LANE_DOUBLES);
	RCARVE(m->a.unit, double, stepRows*20);
	RCARVE(m->a.arbTmp, double, 4*(size_t)d->arbCap);
	RCARVE(m->a.srows, cpgRow, segRows);
	RCARVE(m->a.sbodies, double, (size_t)K*nb*8);
	RCARVE(m->app, double, segRows*(size_t)iters*2*14);     /* AdjApp: 14 doubles */
	return total;
}
#undef RCARVE

/* A segment tape of at least rowCap rows (the kept one if it fits). */
static int seg_alloc(const cpgSet *d, SegTape *sg, int K, size_t rowCap)
{
	if(sg->block && sg->t.K == K && (size_t)sg->t.rowCap >= rowCap) return 1;
	if(rowCap > 0x7fffffffULL/4){ set_error(CP_GPU_ERR_OVERFLOW, "rollout: tape too large"); return 0; }
	if(sg->block) cudaFree(sg->block);
	memset(sg, 0, sizeof(*sg));
	size_t bytes = seg_carve(d, &sg->t, NULL, K, rowCap);
	if(!cuda_ok(cudaMalloc(&sg->block, bytes), "cudaMalloc rollout tape")){ sg->block = NULL; return 0; }
	seg_carve(d, &sg->t, (char *)sg->block, K, rowCap);
	sg->bytes = bytes;
	return 1;
}

/* The reverse pass's scratch, at least segRows x stepRows; `keep` copies
 * the adjoint state of a pass in progress into a larger one. */
static int adj_ensure(const cpgSet *d, AdjMem *m, int K, size_t segRows, size_t stepRows, int iters, int keep)
{
	if(m->block && m->K == K && m->iters == iters && m->segRows >= segRows && m->stepRows >= stepRows) return 1;
	if(segRows < m->segRows) segRows = m->segRows;
	if(stepRows < m->stepRows) stepRows = m->stepRows;
	if(segRows > 0x7fffffffULL/(size_t)(2*iters + 2)){ set_error(CP_GPU_ERR_OVERFLOW, "rollout: tape too large"); return 0; }
	AdjMem n;
	memset(&n, 0, sizeof(n));
	size_t bytes = adj_carve(d, &n, NULL, K, segRows, stepRows, iters);
	if(!cuda_ok(cudaMalloc(&n.block, bytes), "cudaMalloc rollout scratch")) return 0;
	adj_carve(d, &n, (char *)n.block, K, segRows, stepRows, iters);
	n.bytes = bytes; n.segRows = segRows; n.stepRows = stepRows; n.K = K; n.iters = iters;
	if(m->block){
		if(keep){
			cudaStream_t st = lib_stream();
			size_t nb = (size_t)d->totalBodies, ns = (size_t)d->totalShapes;
			cudaMemcpyAsync(n.a.body, m->a.body, sizeof(double)*9*nb, cudaMemcpyDeviceToDevice, st);
			cudaMemcpyAsync(n.a.arb, m->a.arb, sizeof(double)*4*(size_t)d->arbCap, cudaMemcpyDeviceToDevice, st);
			cudaMemcpyAsync(n.a.gMinv, m->a.gMinv, sizeof(double)*nb, cudaMemcpyDeviceToDevice, st);
			cudaMemcpyAsync(n.a.gE, m->a.gE, sizeof(double)*ns, cudaMemcpyDeviceToDevice, st);
			cudaMemcpyAsync(n.a.gU, m->a.gU, sizeof(double)*ns, cudaMemcpyDeviceToDevice, st);
			cudaStreamSynchronize(st);
		}
		cudaFree(m->block);
	}
	*m = n;
	return 1;
}

int cpGpuDebugRolloutTimes(cpGpuBatch *b, double *out)
{
	if(!b || !b->roll || !out) return 0;
	Rollout *r = b->roll;
	double tape = (double)r->adj.bytes;
	for(int i = 0; i < r->segCap; i++) tape += (double)r->segs[i].bytes;
	out[0] = r->replayMs; out[1] = r->adjointMs;
	out[2] = tape;
	out[3] = (double)r->ckptCap*(double)b->dev->slabBytes;
	return 4;
}

/* The iteration count shared by every space of the batch, or -1. */
static int rollout_iterations(DevSet *ds)
{
	int iters = ds->nspaces ? ds->spaces[0]->iterations : 0;
	for(int w = 1; w < ds->nspaces; w++) if(ds->spaces[w]->iterations != iters) return -1;
	return iters;
}

/* Rows to provide for K steps: the largest need seen, or twice the solved
 * arbiters of the latest step plus the joints plus one per shape. */
static size_t rollout_row_estimate(DevSet *ds, Rollout *r, int K)
{
	check_stats(ds);
	size_t est = (size_t)K*(2*(size_t)(ds->hstats[5] > 0 ? ds->hstats[5] : 0) + (size_t)ds->d.totalCons +
		(size_t)ds->d.totalShapes + 1024);
	return r->rowEst > est ? r->rowEst : est;
}

/* Start recording segment `seg` of the forward into its light tape. */
static void seg_begin(DevSet *ds, Rollout *r, int seg)
{
	cpgSet *d = &ds->d;
	SegTape *sg = &r->segs[seg];
	sg->recorded = 0;
	int err0 = g_error;
	if(!seg_alloc(d, sg, r->K, rollout_row_estimate(ds, r, r->K))){
		/* no room: the reverse pass replays the segment from its checkpoint */
		(void)cudaGetLastError();
		g_error = err0;
		return;
	}
	cudaMemsetAsync(sg->t.cursor, 0, sizeof(int)*4, lib_stream());
	d->tape = sg->t;
	d->tape.on = 1;
}

/* End of a segment's recording: it is kept unless it overflowed (then the
 * reverse pass replays it, into a larger tape) or holds joints. */
static void seg_finish(DevSet *ds, Rollout *r, int seg, int len)
{
	cpgSet *d = &ds->d;
	if(!d->tape.on) return;
	d->tape.on = 0;
	SegTape *sg = &r->segs[seg];
	cudaStream_t st = lib_stream();
	int W = ds->nspaces;
	int cur[4] = {0, 0, 0, 0};
	int *off = HALLOC(int, (size_t)len*(W + 1));
	int ok = cuda_ok(cudaMemcpyAsync(cur, sg->t.cursor, sizeof(cur), cudaMemcpyDeviceToHost, st), "tape cursor");
	ok &= cuda_ok(cudaMemcpyAsync(off, sg->t.rowOff, sizeof(int)*(size_t)len*(W + 1), cudaMemcpyDeviceToHost, st), "tape offsets");
	cudaStreamSynchronize(st);
	size_t need = (size_t)cur[0] + (size_t)cur[0]/4 + 1024;
	if(need > r->rowEst) r->rowEst = need;
	if(ok && !cur[2] && !(cur[3] & 1)){
		int mx = 0;
		for(int t = 0; t < len; t++){
			int rows = off[(size_t)t*(W + 1) + W] - off[(size_t)t*(W + 1)];
			if(rows > mx) mx = rows;
		}
		sg->maxStepRows = mx;
		sg->rowsUsed = cur[0];
		sg->recorded = 1;
	}
	free(off);
	memset(&d->tape, 0, sizeof(d->tape));
}

int cpGpuRolloutForward(cpGpuBatch *b, cpFloat dt, int steps, int checkpoint)
{
	if(steps < 1 || checkpoint < 1 || !(dt > 0.0)){ set_error(CP_GPU_ERR_ARGUMENT, "rollout: steps, checkpoint and dt must be positive"); return -1; }
	if(!batch_ready(b)) return -1;
	DevSet *ds = b->dev;
	if(!b->roll) b->roll = (Rollout *)calloc(1, sizeof(Rollout));
	Rollout *r = b->roll;
	if(r->K != checkpoint) r->rowEst = 0;
	r->steps = steps; r->K = checkpoint; r->dt = dt;
	r->nckpt = (steps + checkpoint - 1)/checkpoint;
	free(r->stamps); free(r->currDt);
	r->stamps = HALLOC(unsigned, (size_t)r->nckpt*ds->nspaces);
	r->currDt = HALLOC(double, (size_t)r->nckpt*ds->nspaces);
	if(r->ckptCap < r->nckpt){
		if(r->ckpt) cudaFree(r->ckpt);
		r->ckpt = NULL; r->ckptCap = 0;
		if(!cuda_ok(cudaMalloc((void **)&r->ckpt, (size_t)r->nckpt*ds->slabBytes), "cudaMalloc checkpoints")){
			r->ckpt = NULL;
			set_error(CP_GPU_ERR_OVERFLOW, "rollout: no device memory for %d checkpoints of %zu bytes", r->nckpt, ds->slabBytes);
			return -1;
		}
		r->ckptCap = r->nckpt;
	}
	if(r->segCap < r->nckpt){
		SegTape *ns = (SegTape *)calloc((size_t)r->nckpt, sizeof(SegTape));
		if(r->segs) memcpy(ns, r->segs, sizeof(SegTape)*(size_t)r->segCap);
		free(r->segs);
		r->segs = ns;
		r->segCap = r->nckpt;
	}
	for(int i = 0; i < r->segCap; i++) r->segs[i].recorded = 0;
	double *dts = (double *)malloc(sizeof(double)*(size_t)b->n);
	for(int i = 0; i < b->n; i++) dts[i] = dt;
	int record = rollout_iterations(ds) > 0 && g_rollout_record;
	int rc = 0, seg = -1;
	for(int s = 0; s < steps && rc == 0; s++){
		if(s % checkpoint == 0){
			if(seg >= 0) seg_finish(ds, r, seg, checkpoint);
			seg = s/checkpoint;
			rollout_save(b, seg);
			if(record) seg_begin(ds, r, seg);
		}
		if(ds->d.tape.on) ds->d.tape.step = s - seg*checkpoint;
		rc = devset_step(ds, dts, NULL);
	}
	if(seg >= 0){
		if(rc == 0) seg_finish(ds, r, seg, steps - seg*checkpoint);
		else { ds->d.tape.on = 0; memset(&ds->d.tape, 0, sizeof(ds->d.tape)); }
	}
	free(dts);
	return rc;
}

/* Replays segment `seg` from its checkpoint with full recording (the light
 * tape and the per-iteration records), growing the tape on overflow. */
static int seg_replay(DevSet *ds, Rollout *r, int seg, int len, const double *dts, int iters)
{
	cpgSet *d = &ds->d;
	cudaStream_t st = lib_stream();
	int W = ds->nspaces;
	SegTape *sg = &r->segs[seg];
	for(int attempt = 0; attempt < 4; attempt++){
		size_t rowCap = rollout_row_estimate(ds, r, r->K);
		if(!seg_alloc(d, sg, r->K, rowCap)) return 0;
		if(!adj_ensure(d, &r->adj, r->K, (size_t)sg->t.rowCap, (size_t)sg->t.rowCap, iters, 1)) return 0;
		rollout_restore_from(ds, r->ckpt + (size_t)seg*ds->slabBytes, r->stamps + (size_t)seg*W, r->currDt + (size_t)seg*W);
		cudaMemsetAsync(sg->t.cursor, 0, sizeof(int)*4, st);
		d->tape = sg->t;
		d->tape.app = r->adj.app;
		d->tape.on = 1;
		int ok = 1;
		for(int t = 0; t < len && ok; t++){
			d->tape.step = t;
			if(devset_step(ds, dts, NULL) != 0) ok = 0;
		}
		d->tape.on = 0;
		if(!ok) return 0;
		int cur[4];
		cuda_ok(cudaMemcpyAsync(cur, sg->t.cursor, sizeof(cur), cudaMemcpyDeviceToHost, st), "tape cursor");
		cudaStreamSynchronize(st);
		if(cur[3] & 1){ set_error(CP_GPU_ERR_UNSUPPORTED, "rollout: constraints are not differentiated"); return 0; }
		size_t need = (size_t)cur[0] + (size_t)cur[0]/4 + 1024;
		if(!cur[2]) return 1;
		if(need > r->rowEst) r->rowEst = need;
	}
	set_error(CP_GPU_ERR_OVERFLOW, "rollout: tape overflow");
	return 0;
}

int cpGpuRolloutBackward(cpGpuBatch *b, const cpFloat *dLdp, cpFloat *dLdv0, cpFloat *dLdw0, cpFloat *dLdm, cpFloat *dLde, cpFloat *dLdu)
{
	if(!dLdp){ set_error(CP_GPU_ERR_ARGUMENT, "rollout: dLdp is required"); return -1; }
	return cpGpuRolloutBackwardFull(b, dLdp, NULL, NULL, NULL, NULL, NULL, dLdv0, dLdw0, dLdm, dLde, dLdu);
}

int cpGpuRolloutBackwardFull(cpGpuBatch *b, const cpFloat *dLdp, const cpFloat *dLda, const cpFloat *dLdv, const cpFloat *dLdw,
	cpFloat *dLdp0, cpFloat *dLda0, cpFloat *dLdv0, cpFloat *dLdw0, cpFloat *dLdm, cpFloat *dLde, cpFloat *dLdu)
{
	if(!b || !b->dev || !b->roll || !b->roll->segs){ set_error(CP_GPU_ERR_ARGUMENT, "rollout: no forward rollout to reverse"); return -1; }
	DevSet *ds = b->dev;
	cpgSet *d = &ds->d;
	Rollout *r = b->roll;
	cudaStream_t st = lib_stream();
	int W = ds->nspaces, K = r->K;
	int iters = rollout_iterations(ds);
	if(iters < 0){
		set_error(CP_GPU_ERR_UNSUPPORTED, "rollout: all spaces of the batch need the same iteration count");
		return -1;
	}
	/* the state after the forward, restored at the end (replays move it) */
	if(!r->fin && !cuda_ok(cudaMalloc((void **)&r->fin, ds->slabBytes), "cudaMalloc final state")){ r->fin = NULL; return -1; }
	char *fin = r->fin;
	cuda_ok(cudaMemcpyAsync(fin, ds->slab, ds->slabBytes, cudaMemcpyDeviceToDevice, st), "save final state");
	unsigned *finStamp = HALLOC(unsigned, W);
	double *finDt = HALLOC(double, W);
	for(int w = 0; w < W; w++){ finStamp[w] = ds->spaces[w]->stamp; finDt[w] = ds->spaces[w]->curr_dt; }

	/* scratch for the largest segment and step */
	size_t segRows = 0, stepRows = 0;
	int missing = 0;
	for(int i = 0; i < r->nckpt; i++){
		SegTape *sg = &r->segs[i];
		if(sg->recorded){
			if((size_t)sg->rowsUsed > segRows) segRows = (size_t)sg->rowsUsed;
			if((size_t)sg->maxStepRows > stepRows) stepRows = (size_t)sg->maxStepRows;
		} else missing = 1;
	}
	if(missing){
		size_t est = rollout_row_estimate(ds, r, K);
		if(est > segRows) segRows = est;
		stepRows = segRows;
	}
	int rc = -1;
	double *h = NULL;
	if(!adj_ensure(d, &r->adj, K, segRows, stepRows, iters, 0)) goto done;

	/* seeds: the loss's gradient with respect to the final state (absent
	 * arrays are zero); the bias velocities end every step at zero */
	{
		cpgAdj *A = &r->adj.a;
		size_t nbd = 9*(size_t)d->totalBodies;
		h = HALLOC(double, nbd);
		int idx = 0;
		for(int w = 0; w < W; w++){
			cpSpace *sp = ds->spaces[w];
			for(int i = 0; i < sp->ndyn; i++, idx++){
				size_t g = (size_t)ds->hworld[w].bodyOff + i;
				if(dLdp){ h[9*g] = dLdp[2*idx]; h[9*g + 1] = dLdp[2*idx + 1]; }
				if(dLda) h[9*g + 2] = dLda[idx];
				if(dLdv){ h[9*g + 3] = dLdv[2*idx]; h[9*g + 4] = dLdv[2*idx + 1]; }
				if(dLdw) h[9*g + 5] = dLdw[idx];
			}
		}
		cuda_ok(cudaMemcpyAsync(A->body, h, sizeof(double)*nbd, cudaMemcpyHostToDevice, st), "seed");
		cudaMemsetAsync(A->arb, 0, sizeof(double)*4*(size_t)d->arbCap, st);
		cudaMemsetAsync(A->gMinv, 0, sizeof(double)*(size_t)d->totalBodies, st);
		cudaMemsetAsync(A->gE, 0, sizeof(double)*(size_t)d->totalShapes, st);
		cudaMemsetAsync(A->gU, 0, sizeof(double)*(size_t)d->totalShapes, st);
	}
	{
		double *dts = (double *)malloc(sizeof(double)*(size_t)W);
		for(int i = 0; i < W; i++) dts[i] = r->dt;
		int ok = 1;
		cudaEvent_t ev[3];
		if(g_timing) for(int i = 0; i < 3; i++) cudaEventCreate(&ev[i]);
		r->replayMs = 0.0f; r->adjointMs = 0.0f;
		int *off = HALLOC(int, (size_t)K*(W + 1));
		for(int seg = r->nckpt - 1; seg >= 0 && ok; seg--){
			int first = seg*K, len = (r->steps - first < K) ? r->steps - first : K;
			SegTape *sg = &r->segs[seg];
			if(g_timing) cudaEventRecord(ev[0], st);
			int replayed = 0;
			if(!sg->recorded){
				if(!seg_replay(ds, r, seg, len, dts, iters)){ ok = 0; break; }
				replayed = 1;
			} else {
				/* the solver iterations of the segment's steps, from the
				 * forward's recording, in one launch */
				d->tape = sg->t;
				d->tape.app = r->adj.app;
				d->tape.on = 0;
				if(cpg_launch_replay_solve(d, &r->adj.a, len, st) != 0){ set_error(CP_GPU_ERR_CUDA, "replay solve launch failed"); ok = 0; break; }
			}
			if(g_timing) cudaEventRecord(ev[1], st);
			d->tape = sg->t;
			d->tape.app = r->adj.app;
			d->tape.on = 0;
			/* a replay claims table slots of its own for the arbiters it
			 * creates: the carried impulse adjoints, in the next
			 * checkpoint's (the forward's) numbering, move to the replay's */
			if(replayed && seg + 1 < r->nckpt){
				const char *next = r->ckpt + (size_t)(seg + 1)*ds->slabBytes + ((const char *)d->keys - (const char *)ds->slab);
				if(cpg_launch_adjoint_remap(d, &r->adj.a, next, st) != 0){ set_error(CP_GPU_ERR_CUDA, "adjoint launch failed"); ok = 0; break; }
			}
			cuda_ok(cudaMemcpyAsync(off, sg->t.rowOff, sizeof(int)*(size_t)len*(W + 1), cudaMemcpyDeviceToHost, st), "tape offsets");
			cudaStreamSynchronize(st);
			for(int t = len - 1; t >= 0 && ok; t--){
				int rows = off[(size_t)t*(W + 1) + W] - off[(size_t)t*(W + 1)];
				if((size_t)rows > r->adj.stepRows){ set_error(CP_GPU_ERR_OVERFLOW, "rollout: step scratch too small"); ok = 0; break; }
				if(cpg_launch_adjoint(d, &r->adj.a, t, rows, st) != 0){ set_error(CP_GPU_ERR_CUDA, "adjoint launch failed"); ok = 0; }
			}
			if(ok){
				int cur[4] = {0, 0, 0, 0};
				cuda_ok(cudaMemcpyAsync(cur, sg->t.cursor, sizeof(cur), cudaMemcpyDeviceToHost, st), "tape cursor");
				cudaStreamSynchronize(st);
				if(cur[3] & 2){ set_error(CP_GPU_ERR_CUDA, "rollout: contact geometry of a recorded step did not match its rows"); ok = 0; }
			}
			if(g_timing){
				float a0 = 0.0f, a1 = 0.0f;
				cudaEventRecord(ev[2], st);
				cudaEventSynchronize(ev[2]);
				cudaEventElapsedTime(&a0, ev[0], ev[1]);
				cudaEventElapsedTime(&a1, ev[1], ev[2]);
				r->replayMs += a0; r->adjointMs += a1;
			}
			/* a replayed tape is not the forward's any more */
			if(replayed) sg->recorded = 0;
		}
		free(off);
		free(dts);
		if(g_timing) for(int i = 0; i < 3; i++) cudaEventDestroy(ev[i]);
		if(ok){
			/* gather: dL/dv0, dL/dw0 from the body adjoints, dL/dm = -dL/d(1/m) / m^2 */
			cpgAdj *A = &r->adj.a;
			size_t nbd = 9*(size_t)d->totalBodies;
			double *gm = HALLOC(double, d->totalBodies), *minv = HALLOC(double, d->totalBodies);
			double *ge = HALLOC(double, d->totalShapes), *gu = HALLOC(double, d->totalShapes);
			ok &= cuda_ok(cudaMemcpyAsync(h, A->body, sizeof(double)*nbd, cudaMemcpyDeviceToHost, st), "gradients");
			ok &= cuda_ok(cudaMemcpyAsync(gm, A->gMinv, sizeof(double)*(size_t)d->totalBodies, cudaMemcpyDeviceToHost, st), "gradients");
			ok &= cuda_ok(cudaMemcpyAsync(minv, d->minv, sizeof(double)*(size_t)d->totalBodies, cudaMemcpyDeviceToHost, st), "gradients");
			ok &= cuda_ok(cudaMemcpyAsync(ge, A->gE, sizeof(double)*(size_t)d->totalShapes, cudaMemcpyDeviceToHost, st), "gradients");
			ok &= cuda_ok(cudaMemcpyAsync(gu, A->gU, sizeof(double)*(size_t)d->totalShapes, cudaMemcpyDeviceToHost, st), "gradients");
			cudaStreamSynchronize(st);
			int idx = 0, sidx = 0;
			for(int w = 0; w < W && ok; w++){
				cpSpace *sp = ds->spaces[w];
				for(int i = 0; i < sp->ndyn; i++, idx++){
					size_t g = (size_t)ds->hworld[w].bodyOff + i;
					if(dLdp0){ dLdp0[2*idx] = h[9*g]; dLdp0[2*idx + 1] = h[9*g + 1]; }
					if(dLda0) dLda0[idx] = h[9*g + 2];
					if(dLdv0){ dLdv0[2*idx] = h[9*g + 3]; dLdv0[2*idx + 1] = h[9*g + 4]; }
					if(dLdw0) dLdw0[idx] = h[9*g + 5];
					if(dLdm) dLdm[idx] = -gm[g]*minv[g]*minv[g];
				}
				for(int i = 0; i < sp->nshapes; i++){
					if(!sp->shapes[i]) continue;      /* a removed shape's slot */
					size_t g = (size_t)ds->hworld[w].shapeOff + i;
					if(dLde) dLde[sidx] = ge[g];
					if(dLdu) dLdu[sidx] = gu[g];
					sidx++;
				}
			}
			free(gm); free(minv); free(ge); free(gu);
		}
		rc = ok ? 0 : -1;
	}
done:
	d->tape.on = 0;
	rollout_restore_from(ds, fin, finStamp, finDt);
	cudaStreamSynchronize(st);
	memset(&d->tape, 0, sizeof(d->tape));
	free(finStamp); free(finDt); free(h);
	return rc;
}

/* ====================================================================
 * Creation-time math: chipmunk.c:63-171, 250-274
 * ==================================================================== */
#define PI_ ((cpFloat)3.14159265358979323846264338327950288)

cpFloat cpMomentForCircle(cpFloat m, cpFloat r1, cpFloat r2, cpVect offset) { return m*(0.5*(r1*r1 + r2*r2) + cpvlengthsq(offset)); }
cpFloat cpAreaForCircle(cpFloat r1, cpFloat r2) { return PI_*habs(r1*r1 - r2*r2); }

cpFloat cpMomentForSegment(cpFloat m, cpVect a, cpVect b, cpFloat r)
{
	cpVect offset = cpvlerp(a, b, 0.5);
	cpFloat length = cpvdist(b, a) + 2.0*r;
	return m*((length*length + 4.0*r*r)/12.0 + cpvlengthsq(offset));
}

cpFloat cpAreaForSegment(cpVect a, cpVect b, cpFloat r) { return r*(PI_*r + 2.0*cpvdist(a, b)); }

cpFloat cpMomentForPoly(cpFloat m, int count, const cpVect *verts, cpVect offset, cpFloat r)
{
	(void)r;
	if(count == 2) return cpMomentForSegment(m, verts[0], verts[1], 0.0);
	cpFloat sum1 = 0.0, sum2 = 0.0;
	for(int i = 0; i < count; i++){
		cpVect v1 = cpvadd(verts[i], offset), v2 = cpvadd(verts[(i + 1)%count], offset);
		cpFloat a = cpvcross(v2, v1);
		cpFloat b = cpvdot(v1, v1) + cpvdot(v1, v2) + cpvdot(v2, v2);
		sum1 += a*b;
		sum2 += a;
	}
	return (m*sum1)/(6.0*sum2);
}

cpFloat cpAreaForPoly(const int count, const cpVect *verts, cpFloat r)
{
	cpFloat area = 0.0, perimeter = 0.0;
	for(int i = 0; i < count; i++){
		cpVect v1 = verts[i], v2 = verts[(i + 1)%count];
		area += cpvcross(v1, v2);
		perimeter += cpvdist(v1, v2);
	}
	return r*(PI_*habs(r) + perimeter) + area/2.0;
}

cpVect cpCentroidForPoly(const int count, const cpVect *verts)
{
	cpFloat sum = 0.0;
	cpVect vsum = cpvzero;
	for(int i = 0; i < count; i++){
		cpVect v1 = verts[i], v2 = verts[(i + 1)%count];
		cpFloat cross = cpvcross(v1, v2);
		sum += cross;
		vsum = cpvadd(vsum, cpvmult(cpvadd(v1, v2), cross));
	}
	return cpvmult(vsum, 1.0/(3.0*sum));
}

cpFloat cpMomentForBox(cpFloat m, cpFloat width, cpFloat height) { return m*(width*width + height*height)/12.0; }

cpFloat cpMomentForBox2(cpFloat m, cpBB box)
{
	cpFloat width = box.r - box.l, height = box.t - box.b;
	cpVect offset = cpvmult(cpv(box.l + box.r, box.b + box.t), 0.5);
	return cpMomentForBox(m, width, height) + m*cpvlengthsq(offset);
}

/* QuickHull with in-place partitioning (chipmunk.c:178-274); the output
 * order matters because vertex indices feed contact feature ids. */
static void qh_swap(cpVect *a, cpVect *b) { cpVect t = *a; *a = *b; *b = t; }

static int qh_partition(cpVect *verts, int count, cpVect a, cpVect b, cpFloat tol)
{
	if(count == 0) return 0;
	cpFloat best = 0;
	int pivot = 0;
	cpVect delta = cpvsub(b, a);
	cpFloat valueTol = tol*cpvlength(delta);
	int head = 0;
	for(int tail = count - 1; head <= tail;){
		cpFloat value = cpvcross(cpvsub(verts[head], a), delta);
		if(value > valueTol){
			if(value > best){ best = value; pivot = head; }
			head++;
		} else {
			qh_swap(&verts[head], &verts[tail]);
			tail--;
		}
	}
	if(pivot != 0) qh_swap(&verts[0], &verts[pivot]);
	return head;
}

static int qh_reduce(cpFloat tol, cpVect *verts, int count, cpVect a, cpVect pivot, cpVect b, cpVect *result)
{
	if(count < 0) return 0;
	if(count == 0){ result[0] = pivot; return 1; }
	int left = qh_partition(verts, count, a, pivot, tol);
	int index = qh_reduce(tol, verts + 1, left - 1, a, verts[0], pivot, result);
	result[index++] = pivot;
	int right = qh_partition(verts + left, count - left, pivot, b, tol);
	return index + qh_reduce(tol, verts + left + 1, right - 1, pivot, verts[left], b, result + index);
}

int cpConvexHull(int count, const cpVect *verts, cpVect *result, int *first, cpFloat tol)
{
	if(verts != result) memcpy(result, verts, (size_t)count*sizeof(cpVect));
	int start = 0, end = 0;
	cpVect lo = verts[0], hi = lo;
	for(int i = 1; i < count; i++){
		cpVect v = verts[i];
		if(v.x < lo.x || (v.x == lo.x && v.y < lo.y)){ lo = v; start = i; }
		else if(v.x > hi.x || (v.x == hi.x && v.y > hi.y)){ hi = v; end = i; }
	}
	if(start == end){
		if(first) *first = 0;
		return 1;
	}
	qh_swap(&result[0], &result[start]);
	qh_swap(&result[1], &result[end == 0 ? start : end]);
	cpVect a = result[0], b = result[1];
	if(first) *first = start;
	return qh_reduce(tol, result + 2, count - 2, a, b, a, result + 1) + 1;
}

/* ====================================================================
 * Bodies: cpBody.c
 * ==================================================================== */
static void set_transform_(cpBody *b, cpVect p, cpFloat a)
{
	/* cpBody.c:347-357 */
	cpVect rot = cpvforangle(a);
	cpVect c = b->cog;
	b->transform = cpTransformNewTranspose(rot.x, -rot.y, p.x - (c.x*rot.x - c.y*rot.y),
		rot.y, rot.x, p.y - (c.x*rot.y + c.y*rot.x));
}

/* Read access: make the host copy current first.  After a step only this
 * body is unpacked from the staging block (when it is one of the space's
 * device bodies); anything else brings all of them. */
static inline const cpBody *rd(const cpBody *b)
{
	cpSpace *sp = b->space;
	if(!sp || !sp->dev) return b;
	if(sp->hostStale) space_download(sp);
	DevSet *ds = sp->dev;
	if(ds->structStale && b->pullGen != ds->pullGen && !unpack_one(ds, sp, (cpBody *)b)) space_pull(sp);
	return b;
}
/* Write access: pull, then mark the space's bodies for upload. */
static inline cpBody *wr(cpBody *b)
{
	if(b->space){ space_pull(b->space); b->space->bodyDirty = 1; b->space->editGen++; }
	return b;
}

static void body_init_(cpBody *b, cpFloat m, cpFloat i)
{
	memset(b, 0, sizeof(*b));
	b->velocity_func = cpBodyUpdateVelocity;
	b->position_func = cpBodyUpdatePosition;
	b->index = -1;
	b->m = m; b->m_inv = (m == 0.0 ? INF_ : 1.0/m);
	b->i = i; b->i_inv = (i == 0.0 ? INF_ : 1.0/i);
	set_transform_(b, b->p, 0.0);
}

cpBody *cpBodyNew(cpFloat mass, cpFloat moment)
{
	ASSERT_HARD(0.0 <= mass && mass < INF_, "Mass must be positive and finite.");
	ASSERT_HARD(moment >= 0.0, "Moment of Inertia must be positive.");
	cpBody *b = (cpBody *)calloc(1, sizeof(cpBody));
	body_init_(b, mass, moment);
	return b;
}

static void make_static_(cpBody *b)
{
	b->idleTime = INF_;
	b->m = b->i = INF_;
	b->m_inv = b->i_inv = 0.0;
	b->v = cpvzero; b->w = 0.0;
}

cpBody *cpBodyNewStatic(void) { cpBody *b = cpBodyNew(0.0, 0.0); make_static_(b); return b; }

cpBody *cpBodyNewKinematic(void)
{
	cpBody *b = cpBodyNew(0.0, 0.0);
	b->m = b->i = INF_;
	b->m_inv = b->i_inv = 0.0;
	return b;
}

void cpBodyFree(cpBody *b) { free(b); }
cpBodyType cpBodyGetType(cpBody *b) { return (cpBodyType)body_type_(b); }
static int space_edit_ok(cpSpace *sp);
static int array_delete_(void **arr, int *n, void *obj);
static void record_op_(cpSpace *sp, int kind, cpShape *s, int isStatic);
static void accumulate_mass_(cpBody *b);

void cpBodySetType(cpBody *b, cpBodyType type)
{
	/* cpBody.c:157-205 */
	int oldType = body_type_(b);
	if(oldType == (int)type) return;
	cpSpace *sp = b->space;
	if(sp) ASSERT_HARD(!sp->locked, "This operation cannot be done safely during a call to cpSpaceStep() or during a query. Put these calls into a post-step callback.");
	if(sp && !space_edit_ok(sp)) return;
	if(sp) sp->bodyDirty = 1;
	b->idleTime = (type == CP_BODY_TYPE_STATIC ? INF_ : 0.0);
	if(type == CP_BODY_TYPE_DYNAMIC){
		b->m = b->i = 0.0;
		b->m_inv = b->i_inv = INF_;
		accumulate_mass_(b);
	} else {
		b->m = b->i = INF_;
		b->m_inv = b->i_inv = 0.0;
		b->v = cpvzero;
		b->w = 0.0;
	}
	if(!sp) return;
	/* activated with its new type (a no-op unless it turned dynamic) */
	if(oldType != CP_BODY_TYPE_STATIC) cpBodyActivate(b);
	/* the body changes array (dynamic and kinematic bodies share one), and
	 * its shapes change index: each leaves one tree and enters the other
	 * with its cached box, in shape-list order */
	int fromStatic = (oldType == CP_BODY_TYPE_STATIC), toStatic = (type == CP_BODY_TYPE_STATIC);
	if(fromStatic != toStatic){
		if(fromStatic){
			array_delete_((void **)sp->stat, &sp->nstat, b);
			push_((void ***)&sp->dyn, &sp->ndyn, &sp->capdyn, b);
		} else {
			array_delete_((void **)sp->dyn, &sp->ndyn, b);
			push_((void ***)&sp->stat, &sp->nstat, &sp->capstat, b);
		}
		for(cpShape *s = b->shapeList; s; s = s->next){
			record_op_(sp, CPG_OP_REMOVE, s, fromStatic);
			record_op_(sp, CPG_OP_INSERT, s, toStatic);
		}
	}
}
cpSpace *cpBodyGetSpace(const cpBody *b) { return b->space; }
cpFloat cpBodyGetMass(const cpBody *b) { return b->m; }
cpFloat cpBodyGetMoment(const cpBody *b) { return b->i; }

void cpBodySetMass(cpBody *b, cpFloat m)
{
	ASSERT_HARD(body_type_(b) == CP_BODY_TYPE_DYNAMIC, "You cannot set the mass of kinematic or static bodies.");
	ASSERT_HARD(0.0 <= m && m < INF_, "Mass must be positive and finite.");
	cpBodyActivate(b);
	wr(b); b->m = m; b->m_inv = (m == 0.0 ? INF_ : 1.0/m);
}

void cpBodySetMoment(cpBody *b, cpFloat i)
{
	ASSERT_HARD(i >= 0.0, "Moment of Inertia must be positive.");
	cpBodyActivate(b);
	wr(b); b->i = i; b->i_inv = (i == 0.0 ? INF_ : 1.0/i);
}

cpVect cpBodyGetRotation(const cpBody *b) { rd(b); return cpv(b->transform.a, b->transform.b); }
cpVect cpBodyGetPosition(const cpBody *b) { rd(b); return cpTransformPoint(b->transform, cpvzero); }

void cpBodySetPosition(cpBody *b, cpVect pos)
{
	/* cpBody.c:374-382 */
	cpBodyActivate(b);
	wr(b);
	cpVect p = b->p = cpvadd(cpTransformVect(b->transform, b->cog), pos);
	set_transform_(b, p, b->a);
}

cpVect cpBodyGetCenterOfGravity(const cpBody *b) { return b->cog; }
void cpBodySetCenterOfGravity(cpBody *b, cpVect cog) { cpBodyActivate(b); wr(b); b->cog = cog; }
cpVect cpBodyGetVelocity(const cpBody *b) { rd(b); return b->v; }
void cpBodySetVelocity(cpBody *b, cpVect v) { cpBodyActivate(b); wr(b); b->v = v; }
cpVect cpBodyGetForce(const cpBody *b) { rd(b); return b->f; }
void cpBodySetForce(cpBody *b, cpVect f) { cpBodyActivate(b); wr(b); b->f = f; }
cpFloat cpBodyGetAngle(const cpBody *b) { rd(b); return b->a; }
void cpBodySetAngle(cpBody *b, cpFloat a) { cpBodyActivate(b); wr(b); b->a = a; set_transform_(b, b->p, a); }
cpFloat cpBodyGetAngularVelocity(const cpBody *b) { rd(b); return b->w; }
void cpBodySetAngularVelocity(cpBody *b, cpFloat w) { cpBodyActivate(b); wr(b); b->w = w; }
cpFloat cpBodyGetTorque(const cpBody *b) { rd(b); return b->t; }
void cpBodySetTorque(cpBody *b, cpFloat t) { cpBodyActivate(b); wr(b); b->t = t; }
cpDataPointer cpBodyGetUserData(const cpBody *b) { return b->userData; }
void cpBodySetUserData(cpBody *b, cpDataPointer d) { b->userData = d; }
void cpBodySetVelocityUpdateFunc(cpBody *b, cpBodyVelocityFunc f) { b->velocity_func = f; }
void cpBodySetPositionUpdateFunc(cpBody *b, cpBodyPositionFunc f) { b->position_func = f; }
cpVect cpBodyLocalToWorld(const cpBody *b, const cpVect p) { rd(b); return cpTransformPoint(b->transform, p); }
cpVect cpBodyWorldToLocal(const cpBody *b, const cpVect p) { rd(b); return cpTransformPoint(rigid_inverse(b->transform), p); }

void cpBodyApplyForceAtWorldPoint(cpBody *b, cpVect force, cpVect point)
{
	cpBodyActivate(b);
	wr(b);
	b->f = cpvadd(b->f, force);
	cpVect r = cpvsub(point, cpTransformPoint(b->transform, b->cog));
	b->t += cpvcross(r, force);
}

void cpBodyApplyForceAtLocalPoint(cpBody *b, cpVect force, cpVect point)
{
	rd(b);
	cpBodyApplyForceAtWorldPoint(b, cpTransformVect(b->transform, force), cpTransformPoint(b->transform, point));
}

void cpBodyApplyImpulseAtWorldPoint(cpBody *b, cpVect j, cpVect point)
{
	cpBodyActivate(b);
	wr(b);
	cpVect r = cpvsub(point, cpTransformPoint(b->transform, b->cog));
	b->v = cpvadd(b->v, cpvmult(j, b->m_inv));
	b->w += b->i_inv*cpvcross(r, j);
}

void cpBodyApplyImpulseAtLocalPoint(cpBody *b, cpVect j, cpVect point)
{
	rd(b);
	cpBodyApplyImpulseAtWorldPoint(b, cpTransformVect(b->transform, j), cpTransformPoint(b->transform, point));
}

cpVect cpBodyGetVelocityAtWorldPoint(const cpBody *b, cpVect point)
{
	rd(b);
	cpVect r = cpvsub(point, cpTransformPoint(b->transform, b->cog));
	return cpvadd(b->v, cpvmult(cpvperp(r), b->w));
}

cpVect cpBodyGetVelocityAtLocalPoint(const cpBody *b, cpVect point)
{
	rd(b);
	cpVect r = cpTransformVect(b->transform, cpvsub(point, b->cog));
	return cpvadd(b->v, cpvmult(cpvperp(r), b->w));
}

cpFloat cpBodyKineticEnergy(const cpBody *b)
{
	rd(b);
	cpFloat vsq = cpvdot(b->v, b->v), wsq = b->w*b->w;
	return (vsq ? vsq*b->m : 0.0) + (wsq ? wsq*b->i : 0.0);
}

/* The reference integrators, for programs that call them directly; the
 * device step runs its own copies of these (cpBody.c:493-522). */
void cpBodyUpdateVelocity(cpBody *b, cpVect gravity, cpFloat damping, cpFloat dt)
{
	wr(b);
	if(body_type_(b) == CP_BODY_TYPE_KINEMATIC) return;
	b->v = cpvadd(cpvmult(b->v, damping), cpvmult(cpvadd(gravity, cpvmult(b->f, b->m_inv)), dt));
	b->w = b->w*damping + b->t*b->i_inv*dt;
	b->f = cpvzero;
	b->t = 0.0;
}

void cpBodyUpdatePosition(cpBody *b, cpFloat dt)
{
	wr(b);
	cpVect p = b->p = cpvadd(b->p, cpvmult(cpvadd(b->v, b->v_bias), dt));
	cpFloat a = b->a = b->a + (b->w + b->w_bias)*dt;
	set_transform_(b, p, a);
	b->v_bias = cpvzero;
	b->w_bias = 0.0;
}

void cpBodyEachShape(cpBody *b, cpBodyShapeIteratorFunc func, void *data)
{
	cpShape *s = b->shapeList;
	while(s){ cpShape *next = s->next; func(b, s, data); s = next; }
}

static inline cpConstraint *cons_next_(cpConstraint *c, cpBody *b) { return (c->a == b ? c->next_a : c->next_b); }

void cpBodyEachConstraint(cpBody *b, cpBodyConstraintIteratorFunc func, void *data)
{
	cpConstraint *c = b->constraintList;
	while(c){ cpConstraint *next = cons_next_(c, b); func(b, c, data); c = next; }
}

/* cpBody.c:206-239 */
static void accumulate_mass_(cpBody *b)
{
	if(b == NULL || body_type_(b) != CP_BODY_TYPE_DYNAMIC) return;
	wr(b);
	b->m = b->i = 0.0;
	b->cog = cpvzero;
	cpVect pos = cpBodyGetPosition(b);
	for(cpShape *s = b->shapeList; s; s = s->next){
		cpFloat m = s->mass_m;
		if(m > 0.0){
			cpFloat msum = b->m + m;
			b->i += m*s->mass_i + cpvdistsq(b->cog, s->mass_cog)*(m*b->m)/msum;
			b->cog = cpvlerp(b->cog, s->mass_cog, m/msum);
			b->m = msum;
		}
	}
	b->m_inv = 1.0/b->m;
	b->i_inv = 1.0/b->i;
	cpBodySetPosition(b, pos);
}

/* ====================================================================
 * Shapes: cpShape.c, cpPolyShape.c
 * ==================================================================== */
static cpShape *shape_new_(int kind, cpBody *body, cpFloat mi, cpVect cog, cpFloat area)
{
	cpShape *s = (cpShape *)calloc(1, sizeof(cpShape));
	s->kind = kind;
	s->body = body;
	s->mass_m = 0.0; s->mass_i = mi; s->mass_cog = cog; s->mass_area = area;
	s->filter.group = CP_NO_GROUP;
	s->filter.categories = CP_ALL_CATEGORIES;
	s->filter.mask = CP_ALL_CATEGORIES;
	return s;
}

/* Add-time shape caches: cpShape.c:291-296, 378-405, cpPolyShape.c:39-64 */
static cpBB shape_cache_(cpShape *s, cpTransform t)
{
	cpBB bb;
	if(s->kind == CPG_CIRCLE){
		cpVect c = s->tc = cpTransformPoint(t, s->c);
		bb = cpBBNewForCircle(c, s->r);
	} else if(s->kind == CPG_SEGMENT){
		s->ta = cpTransformPoint(t, s->sa);
		s->tb = cpTransformPoint(t, s->sb);
		s->tn = cpTransformVect(t, s->sn);
		cpFloat l, r, b, tp;
		if(s->ta.x < s->tb.x){ l = s->ta.x; r = s->tb.x; } else { l = s->tb.x; r = s->ta.x; }
		if(s->ta.y < s->tb.y){ b = s->ta.y; tp = s->tb.y; } else { b = s->tb.y; tp = s->ta.y; }
		bb = cpBBNew(l - s->r, b - s->r, r + s->r, tp + s->r);
	} else {
		cpFloat l = INF_, r = -INF_, b = INF_, tp = -INF_;
		for(int i = 0; i < s->count; i++){
			cpVect v = cpTransformPoint(t, s->lv[i]);
			cpVect n = cpTransformVect(t, s->ln[i]);
			s->gv[i] = v; s->gn[i] = n;
			l = hmin(l, v.x); r = hmax(r, v.x);
			b = hmin(b, v.y); tp = hmax(tp, v.y);
		}
		bb = cpBBNew(l - s->r, b - s->r, r + s->r, tp + s->r);
	}
	return (s->bb = bb);
}

/* Device caches are current after a step: copy the space's shape boxes
 * back in one transfer when a box is read. */
static void shapes_pull_(cpSpace *sp)
{
	if(!sp || !sp->dev || !sp->shapesStale) return;
	DevSet *ds = sp->dev;
	int n = sp->nshapes, off = ds->hworld[sp->world].shapeOff;
	double *buf = HALLOC(double, 4*n);
	d2h(buf, ds->d.bbl + off, sizeof(double)*(size_t)n);
	d2h(buf + n, ds->d.bbb + off, sizeof(double)*(size_t)n);
	d2h(buf + 2*n, ds->d.bbr + off, sizeof(double)*(size_t)n);
	d2h(buf + 3*n, ds->d.bbt + off, sizeof(double)*(size_t)n);
	cuda_ok(cudaStreamSynchronize(lib_stream()), "download shape boxes");
	for(int i = 0; i < n; i++) if(sp->shapes[i]) sp->shapes[i]->bb = cpBBNew(buf[i], buf[n + i], buf[2*n + i], buf[3*n + i]);
	free(buf);
	sp->shapesStale = 0;
}

/* The device's whole shape caches (boxes and world geometry) into the
 * host structs, before a rebuild uploads them again: a shape whose body
 * turns static keeps the caches of its last step (the reference updates
 * only dynamic shapes, cpSpaceStep.c:380-382). */
static void shapes_pull_all_(cpSpace *sp)
{
	if(!sp || !sp->dev) return;
	DevSet *ds = sp->dev;
	shapes_pull_(sp);
	const cpgWorld *W = &ds->hworld[sp->world];
	int n = W->nshapes, nv = W->nverts;
	if(n > sp->nshapes) n = sp->nshapes;
	double *buf = HALLOC(double, 6*(size_t)W->nshapes + 4*(size_t)nv);
	const double *src[6] = { ds->d.w0x, ds->d.w0y, ds->d.w1x, ds->d.w1y, ds->d.wnx, ds->d.wny };
	for(int k = 0; k < 6; k++) d2h(buf + (size_t)k*W->nshapes, src[k] + W->shapeOff, sizeof(double)*(size_t)W->nshapes);
	double *vb = buf + 6*(size_t)W->nshapes;
	const double *vsrc[4] = { ds->d.gvx, ds->d.gvy, ds->d.gnx, ds->d.gny };
	for(int k = 0; k < 4; k++) d2h(vb + (size_t)k*nv, vsrc[k] + W->vertOff, sizeof(double)*(size_t)nv);
	int *voff = HALLOC(int, W->nshapes);
	d2h(voff, ds->d.svoff + W->shapeOff, sizeof(int)*(size_t)W->nshapes);
	if(!cuda_ok(cudaStreamSynchronize(lib_stream()), "download shape caches")){ free(buf); free(voff); return; }
	size_t S = (size_t)W->nshapes;
	for(int i = 0; i < n; i++){
		cpShape *sh = sp->shapes[i];
		if(!sh) continue;
		cpVect g0 = cpv(buf[i], buf[S + i]), g1 = cpv(buf[2*S + i], buf[3*S + i]), gn = cpv(buf[4*S + i], buf[5*S + i]);
		if(sh->kind == CPG_CIRCLE){
			sh->tc = g0;
		} else if(sh->kind == CPG_SEGMENT){
			sh->ta = g0; sh->tb = g1; sh->tn = gn;
		} else {
			for(int j = 0; j < sh->count && voff[i] + j < nv; j++){
				size_t v = (size_t)voff[i] + j;
				sh->gv[j] = cpv(vb[v], vb[nv + v]);
				sh->gn[j] = cpv(vb[2*(size_t)nv + v], vb[3*(size_t)nv + v]);
			}
		}
	}
	free(buf); free(voff);
}

static cpBB shape_bb_now_(cpShape *s)
{
	if(s->space) shapes_pull_(s->space);
	return s->bb;
}

cpBB cpShapeCacheBB(cpShape *s) { rd(s->body); return shape_cache_(s, s->body->transform); }
cpBB cpShapeGetBB(const cpShape *s) { return shape_bb_now_((cpShape *)s); }

cpShape *cpCircleShapeNew(cpBody *body, cpFloat radius, cpVect offset)
{
	/* cpShape.c:313-335 */
	cpShape *s = shape_new_(CPG_CIRCLE, body, cpMomentForCircle(1.0, 0.0, radius, cpvzero), offset, cpAreaForCircle(0.0, radius));
	s->c = offset;
	s->r = radius;
	return s;
}

cpShape *cpSegmentShapeNew(cpBody *body, cpVect a, cpVect b, cpFloat r)
{
	/* cpShape.c:470-502 */
	cpShape *s = shape_new_(CPG_SEGMENT, body, cpMomentForBox(1.0, cpvdist(a, b) + 2.0*r, 2.0*r), cpvlerp(a, b, 0.5), cpAreaForSegment(a, b, r));
	s->sa = a; s->sb = b;
	s->sn = cpvrperp(cpvnormalize(cpvsub(b, a)));
	s->r = r;
	return s;
}

void cpSegmentShapeSetNeighbors(cpShape *s, cpVect prev, cpVect next)
{
	s->a_tangent = cpvsub(prev, s->sa);
	s->b_tangent = cpvsub(next, s->sb);
	if(s->space) s->space->shapeDirty = 1;
}

cpShape *cpPolyShapeNewRaw(cpBody *body, int count, const cpVect *verts, cpFloat radius)
{
	/* cpPolyShape.c:147-165, 202-211 */
	cpVect centroid = cpCentroidForPoly(count, verts);
	cpShape *s = shape_new_(CPG_POLY, body, cpMomentForPoly(1.0, count, verts, cpvneg(centroid), radius), centroid, cpAreaForPoly(count, verts, radius));
	s->count = count;
	s->lv = (cpVect *)calloc((size_t)(4*count), sizeof(cpVect));
	s->ln = s->lv + count; s->gv = s->lv + 2*count; s->gn = s->lv + 3*count;
	for(int i = 0; i < count; i++){
		cpVect a = verts[(i - 1 + count)%count], b = verts[i];
		s->lv[i] = b;
		s->ln[i] = cpvnormalize(cpvrperp(cpvsub(b, a)));
	}
	s->r = radius;
	return s;
}

/* chipmunk_unsafe.h: shapes changed in place (cpShape.c:553-604,
 * cpPolyShape.c:287-324).  A shape in a space comes home first: the set is
 * rebuilt with its new geometry (the polygon's vertex layout may change),
 * and the caches update at the next cpShapeUpdate, as in the reference. */
static void unsafe_edit_(cpShape *s)
{
	if(s->space) space_edit_ok(s->space);
}

void cpCircleShapeSetRadius(cpShape *s, cpFloat radius)
{
	ASSERT_HARD(s->kind == CPG_CIRCLE, "Shape is not a circle shape.");
	unsafe_edit_(s);
	s->r = radius;
	cpFloat mass = s->mass_m;
	s->mass_i = cpMomentForCircle(1.0, 0.0, s->r, cpvzero); s->mass_cog = s->c; s->mass_area = cpAreaForCircle(0.0, s->r);
	if(mass > 0.0) accumulate_mass_(s->body);
}

void cpCircleShapeSetOffset(cpShape *s, cpVect offset)
{
	ASSERT_HARD(s->kind == CPG_CIRCLE, "Shape is not a circle shape.");
	unsafe_edit_(s);
	s->c = offset;
	cpFloat mass = s->mass_m;
	s->mass_i = cpMomentForCircle(1.0, 0.0, s->r, cpvzero); s->mass_cog = s->c; s->mass_area = cpAreaForCircle(0.0, s->r);
	if(mass > 0.0) accumulate_mass_(s->body);
}

/* the normal is cpvperp here, not the constructor's cpvrperp (cpShape.c:586) */
void cpSegmentShapeSetEndpoints(cpShape *s, cpVect a, cpVect b)
{
	ASSERT_HARD(s->kind == CPG_SEGMENT, "Shape is not a segment shape.");
	unsafe_edit_(s);
	s->sa = a; s->sb = b;
	s->sn = cpvperp(cpvnormalize(cpvsub(b, a)));
	cpFloat mass = s->mass_m;
	s->mass_i = cpMomentForBox(1.0, cpvdist(s->sa, s->sb) + 2.0*s->r, 2.0*s->r);
	s->mass_cog = cpvlerp(s->sa, s->sb, 0.5); s->mass_area = cpAreaForSegment(s->sa, s->sb, s->r);
	if(mass > 0.0) accumulate_mass_(s->body);
}

void cpSegmentShapeSetRadius(cpShape *s, cpFloat radius)
{
	ASSERT_HARD(s->kind == CPG_SEGMENT, "Shape is not a segment shape.");
	unsafe_edit_(s);
	s->r = radius;
	cpFloat mass = s->mass_m;
	s->mass_i = cpMomentForBox(1.0, cpvdist(s->sa, s->sb) + 2.0*s->r, 2.0*s->r);
	s->mass_cog = cpvlerp(s->sa, s->sb, 0.5); s->mass_area = cpAreaForSegment(s->sa, s->sb, s->r);
	if(mass > 0.0) accumulate_mass_(s->body);
}

void cpPolyShapeSetVertsRaw(cpShape *s, int count, cpVect *verts)
{
	ASSERT_HARD(s->kind == CPG_POLY, "Shape is not a poly shape.");
	unsafe_edit_(s);
	free(s->lv);
	s->count = count;
	s->lv = (cpVect *)calloc((size_t)(4*(count > 0 ? count : 1)), sizeof(cpVect));
	s->ln = s->lv + count; s->gv = s->lv + 2*count; s->gn = s->lv + 3*count;
	for(int i = 0; i < count; i++){
		cpVect a = verts[(i - 1 + count)%count], b = verts[i];
		s->lv[i] = b;
		s->ln[i] = cpvnormalize(cpvrperp(cpvsub(b, a)));
	}
	cpFloat mass = s->mass_m;
	cpVect centroid = cpCentroidForPoly(count, verts);
	s->mass_i = cpMomentForPoly(1.0, count, verts, cpvneg(centroid), s->r);
	s->mass_cog = centroid; s->mass_area = cpAreaForPoly(count, verts, s->r);
	if(mass > 0.0) accumulate_mass_(s->body);
}

void cpPolyShapeSetVerts(cpShape *s, int count, cpVect *verts, cpTransform transform)
{
	cpVect *hull = (cpVect *)malloc((size_t)(count > 0 ? count : 1)*sizeof(cpVect));
	for(int i = 0; i < count; i++) hull[i] = cpTransformPoint(transform, verts[i]);
	int n = cpConvexHull(count, hull, hull, NULL, 0.0);
	cpPolyShapeSetVertsRaw(s, n, hull);
	free(hull);
}

/* the radius alone: the reference leaves the mass properties (cpPolyShape.c:313-324) */
void cpPolyShapeSetRadius(cpShape *s, cpFloat radius)
{
	ASSERT_HARD(s->kind == CPG_POLY, "Shape is not a poly shape.");
	unsafe_edit_(s);
	s->r = radius;
}

/* cpShape.c:87-92, 216-220 */
void cpShapeSetBody(cpShape *s, cpBody *body)
{
	ASSERT_HARD(!(s->prev || (s->body && s->body->shapeList == s)), "You cannot change the body on an active shape. You must remove the shape from the space before changing the body.");
	s->body = body;
}

cpBB cpShapeUpdate(cpShape *s, cpTransform transform) { return shape_cache_(s, transform); }

cpShape *cpPolyShapeNew(cpBody *body, int count, const cpVect *verts, cpTransform transform, cpFloat radius)
{
	cpVect *hull = (cpVect *)malloc((size_t)count*sizeof(cpVect));
	for(int i = 0; i < count; i++) hull[i] = cpTransformPoint(transform, verts[i]);
	int n = cpConvexHull(count, hull, hull, NULL, 0.0);
	cpShape *s = cpPolyShapeNewRaw(body, n, hull, radius);
	free(hull);
	return s;
}

cpShape *cpBoxShapeNew2(cpBody *body, cpBB box, cpFloat radius)
{
	cpVect verts[4] = { cpv(box.r, box.b), cpv(box.r, box.t), cpv(box.l, box.t), cpv(box.l, box.b) };
	return cpPolyShapeNewRaw(body, 4, verts, radius);
}

cpShape *cpBoxShapeNew(cpBody *body, cpFloat width, cpFloat height, cpFloat radius)
{
	cpFloat hw = width/2.0, hh = height/2.0;
	return cpBoxShapeNew2(body, cpBBNew(-hw, -hh, hw, hh), radius);
}

void cpShapeFree(cpShape *s) { if(s){ free(s->lv); free(s); } }
void cpShapeDestroy(cpShape *s);

static inline cpShape *swr(cpShape *s) { cpBodyActivate(s->body); if(s->space){ s->space->shapeDirty = 1; s->space->editGen++; } return s; }

cpSpace *cpShapeGetSpace(const cpShape *s) { return s->space; }
cpBody *cpShapeGetBody(const cpShape *s) { return s->body; }
cpFloat cpShapeGetMass(cpShape *s) { return s->mass_m; }
void cpShapeSetMass(cpShape *s, cpFloat mass) { cpBodyActivate(s->body); s->mass_m = mass; accumulate_mass_(s->body); }
cpFloat cpShapeGetDensity(cpShape *s) { return s->mass_m/s->mass_area; }
void cpShapeSetDensity(cpShape *s, cpFloat d) { cpShapeSetMass(s, d*s->mass_area); }
cpFloat cpShapeGetMoment(cpShape *s) { return s->mass_m*s->mass_i; }
cpFloat cpShapeGetArea(cpShape *s) { return s->mass_area; }
cpVect cpShapeGetCenterOfGravity(cpShape *s) { return s->mass_cog; }
cpBool cpShapeGetSensor(const cpShape *s) { return s->sensor; }
void cpShapeSetSensor(cpShape *s, cpBool v) { swr(s)->sensor = v; }
cpFloat cpShapeGetElasticity(const cpShape *s) { return s->e; }
void cpShapeSetElasticity(cpShape *s, cpFloat e) { ASSERT_HARD(e >= 0.0, "Elasticity must be positive."); swr(s)->e = e; }
cpFloat cpShapeGetFriction(const cpShape *s) { return s->u; }
void cpShapeSetFriction(cpShape *s, cpFloat u) { ASSERT_HARD(u >= 0.0, "Friction must be postive."); swr(s)->u = u; }
cpVect cpShapeGetSurfaceVelocity(const cpShape *s) { return s->surfaceV; }
void cpShapeSetSurfaceVelocity(cpShape *s, cpVect v) { swr(s)->surfaceV = v; }
cpDataPointer cpShapeGetUserData(const cpShape *s) { return s->userData; }
void cpShapeSetUserData(cpShape *s, cpDataPointer d) { s->userData = d; }
cpCollisionType cpShapeGetCollisionType(const cpShape *s) { return s->ctype; }
void cpShapeSetCollisionType(cpShape *s, cpCollisionType t) { cpBodyActivate(s->body); s->ctype = t; if(s->space) s->space->shapeDirty = 1; }
cpShapeFilter cpShapeGetFilter(const cpShape *s) { return s->filter; }
void cpShapeSetFilter(cpShape *s, cpShapeFilter f) { swr(s)->filter = f; }
cpVect cpCircleShapeGetOffset(const cpShape *s) { return s->c; }
cpFloat cpCircleShapeGetRadius(const cpShape *s) { return s->r; }
cpVect cpSegmentShapeGetA(const cpShape *s) { return s->sa; }
cpVect cpSegmentShapeGetB(const cpShape *s) { return s->sb; }
cpVect cpSegmentShapeGetNormal(const cpShape *s) { return s->sn; }
cpFloat cpSegmentShapeGetRadius(const cpShape *s) { return s->r; }
int cpPolyShapeGetCount(const cpShape *s) { return s->count; }
cpVect cpPolyShapeGetVert(const cpShape *s, int i) { ASSERT_HARD(0 <= i && i < s->count, "Index out of range."); return s->lv[i]; }
cpFloat cpPolyShapeGetRadius(const cpShape *s) { return s->r; }

/* ====================================================================
 * Constraints
 * ==================================================================== */
static cpConstraint *cons_new_(int kind, cpBody *a, cpBody *b)
{
	/* cpConstraint.c:37-57; errorBias uses the float expression 1.0f - 0.1f */
	cpConstraint *c = (cpConstraint *)calloc(1, sizeof(cpConstraint));
	c->kind = kind;
	c->a = a; c->b = b;
	c->maxForce = INF_;
	c->errorBias = pow((cpFloat)(1.0f - 0.1f), 60.0);
	c->maxBias = INF_;
	c->collideBodies = cpTrue;
	c->index = -1;
	return c;
}

cpConstraint *cpPivotJointNew2(cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB)
{
	cpConstraint *c = cons_new_(CPG_PIVOT, a, b);
	c->anchorA = anchorA; c->anchorB = anchorB;
	return c;
}

cpConstraint *cpPivotJointNew(cpBody *a, cpBody *b, cpVect pivot)
{
	/* cpPivotJoint.c:110-116 */
	cpVect anchorA = (a ? cpBodyWorldToLocal(a, pivot) : pivot);
	cpVect anchorB = (b ? cpBodyWorldToLocal(b, pivot) : pivot);
	return cpPivotJointNew2(a, b, anchorA, anchorB);
}

cpConstraint *cpPinJointNew(cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB)
{
	/* cpPinJoint.c:92-110 */
	cpConstraint *c = cons_new_(CPG_PIN, a, b);
	c->anchorA = anchorA; c->anchorB = anchorB;
	cpVect p1 = (a ? cpTransformPoint(rd(a)->transform, anchorA) : anchorA);
	cpVect p2 = (b ? cpTransformPoint(rd(b)->transform, anchorB) : anchorB);
	c->dist = cpvlength(cpvsub(p2, p1));
	return c;
}

cpConstraint *cpSlideJointNew(cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB, cpFloat min, cpFloat max)
{
	cpConstraint *c = cons_new_(CPG_SLIDE, a, b);
	c->anchorA = anchorA; c->anchorB = anchorB;
	c->min = min; c->max = max;
	return c;
}

/* Joint records on the device accumulate impulses; refresh them lazily. */
static void joints_pull_(cpSpace *sp)
{
	if(!sp || !sp->dev || !sp->consStale) return;
	DevSet *ds = sp->dev;
	int n = sp->ncons;
	if(n > 0){
		cpgJoint *rec = HALLOC(cpgJoint, n);
		d2h(rec, ds->d.joints + ds->hworld[sp->world].consOff, sizeof(cpgJoint)*(size_t)n);
		cuda_ok(cudaStreamSynchronize(lib_stream()), "download joints");
		for(int i = 0; i < n; i++) sp->cons[i]->rec = rec[i];
		free(rec);
	}
	sp->consStale = 0;
}

static void cons_pull_(cpConstraint *c) { if(c->space) joints_pull_(c->space); }

/* A joint setter's write access; the setters wake both bodies
 * (cpConstraintActivateBodies, chipmunk_private.h:165-170). */
static inline cpConstraint *cwr(cpConstraint *c)
{
	cpBodyActivate(c->a);
	cpBodyActivate(c->b);
	if(c->space){
		joints_pull_(c->space);   /* keep the device-side accumulators */
		c->space->consDirty = 1;
		c->space->editGen++;
	}
	return c;
}

void cpConstraintFree(cpConstraint *c) { free(c); }
cpSpace *cpConstraintGetSpace(const cpConstraint *c) { return c->space; }
cpBody *cpConstraintGetBodyA(const cpConstraint *c) { return c->a; }
cpBody *cpConstraintGetBodyB(const cpConstraint *c) { return c->b; }
cpFloat cpConstraintGetMaxForce(const cpConstraint *c) { return c->maxForce; }
void cpConstraintSetMaxForce(cpConstraint *c, cpFloat v) { ASSERT_HARD(v >= 0.0, "maxForce must be positive."); cwr(c)->maxForce = v; }
cpFloat cpConstraintGetErrorBias(const cpConstraint *c) { return c->errorBias; }
void cpConstraintSetErrorBias(cpConstraint *c, cpFloat v) { ASSERT_HARD(v >= 0.0, "errorBias must be positive."); cwr(c)->errorBias = v; }
cpFloat cpConstraintGetMaxBias(const cpConstraint *c) { return c->maxBias; }
void cpConstraintSetMaxBias(cpConstraint *c, cpFloat v) { ASSERT_HARD(v >= 0.0, "maxBias must be positive."); cwr(c)->maxBias = v; }
cpBool cpConstraintGetCollideBodies(const cpConstraint *c) { return c->collideBodies; }
void cpConstraintSetCollideBodies(cpConstraint *c, cpBool v)
{
	ASSERT_HARD(!c->space || !c->space->dev, "collideBodies must be set before the space is first stepped");
	cpBodyActivate(c->a);
	cpBodyActivate(c->b);
	c->collideBodies = v;
}
void cpConstraintSetPreSolveFunc(cpConstraint *c, cpConstraintPreSolveFunc f) { c->preSolve = f; }
cpConstraintPreSolveFunc cpConstraintGetPreSolveFunc(const cpConstraint *c) { return c->preSolve; }
cpConstraintPostSolveFunc cpConstraintGetPostSolveFunc(const cpConstraint *c) { return c->postSolve; }
void cpConstraintSetPostSolveFunc(cpConstraint *c, cpConstraintPostSolveFunc f) { c->postSolve = f; }
cpDataPointer cpConstraintGetUserData(const cpConstraint *c) { return c->userData; }
void cpConstraintSetUserData(cpConstraint *c, cpDataPointer d) { c->userData = d; }
cpBool cpConstraintIsPivotJoint(const cpConstraint *c) { return c->kind == CPG_PIVOT; }
cpBool cpConstraintIsPinJoint(const cpConstraint *c) { return c->kind == CPG_PIN; }
cpBool cpConstraintIsSlideJoint(const cpConstraint *c) { return c->kind == CPG_SLIDE; }
cpVect cpPivotJointGetAnchorA(const cpConstraint *c) { return c->anchorA; }
cpVect cpPivotJointGetAnchorB(const cpConstraint *c) { return c->anchorB; }
cpVect cpPinJointGetAnchorA(const cpConstraint *c) { return c->anchorA; }
cpVect cpPinJointGetAnchorB(const cpConstraint *c) { return c->anchorB; }
cpFloat cpPinJointGetDist(const cpConstraint *c) { return c->dist; }
cpVect cpSlideJointGetAnchorA(const cpConstraint *c) { return c->anchorA; }
cpVect cpSlideJointGetAnchorB(const cpConstraint *c) { return c->anchorB; }
cpFloat cpSlideJointGetMin(const cpConstraint *c) { return c->min; }
cpFloat cpSlideJointGetMax(const cpConstraint *c) { return c->max; }
/* setters: cpPivotJoint.c:145-165, cpPinJoint.c:148-180, cpSlideJoint.c:158-201
 * (the reference also wakes the bodies; there is no sleeping here) */
void cpPivotJointSetAnchorA(cpConstraint *c, cpVect v) { ASSERT_HARD(c->kind == CPG_PIVOT, "Constraint is not a pivot joint."); cwr(c)->anchorA = v; }
void cpPivotJointSetAnchorB(cpConstraint *c, cpVect v) { ASSERT_HARD(c->kind == CPG_PIVOT, "Constraint is not a pivot joint."); cwr(c)->anchorB = v; }
void cpPinJointSetAnchorA(cpConstraint *c, cpVect v) { ASSERT_HARD(c->kind == CPG_PIN, "Constraint is not a pin joint."); cwr(c)->anchorA = v; }
void cpPinJointSetAnchorB(cpConstraint *c, cpVect v) { ASSERT_HARD(c->kind == CPG_PIN, "Constraint is not a pin joint."); cwr(c)->anchorB = v; }
void cpPinJointSetDist(cpConstraint *c, cpFloat d) { ASSERT_HARD(c->kind == CPG_PIN, "Constraint is not a pin joint."); cwr(c)->dist = d; }
void cpSlideJointSetAnchorA(cpConstraint *c, cpVect v) { ASSERT_HARD(c->kind == CPG_SLIDE, "Constraint is not a slide joint."); cwr(c)->anchorA = v; }
void cpSlideJointSetAnchorB(cpConstraint *c, cpVect v) { ASSERT_HARD(c->kind == CPG_SLIDE, "Constraint is not a slide joint."); cwr(c)->anchorB = v; }
void cpSlideJointSetMin(cpConstraint *c, cpFloat v) { ASSERT_HARD(c->kind == CPG_SLIDE, "Constraint is not a slide joint."); cwr(c)->min = v; }
void cpSlideJointSetMax(cpConstraint *c, cpFloat v) { ASSERT_HARD(c->kind == CPG_SLIDE, "Constraint is not a slide joint."); cwr(c)->max = v; }

cpFloat cpConstraintGetImpulse(cpConstraint *c)
{
	cons_pull_(c);
	if(c->kind == CPG_PIVOT || c->kind == CPG_GROOVE) return cpvlength(cpv(c->rec.jx, c->rec.jy));
	/* the springs report their signed accumulated impulse
	 * (cpDampedSpring.c:79-83, cpDampedRotarySpring.c:74-78) */
	if(c->kind == CPG_DSPRING || c->kind == CPG_DRSPRING) return c->rec.jnAcc;
	return habs(c->rec.jnAcc);
}

/* The remaining joints (constructors: cpGrooveJoint.c:119-132,
 * cpDampedSpring.c:124-140, cpDampedRotarySpring.c:100-115,
 * cpRotaryLimitJoint.c:108-119, cpRatchetJoint.c:111-123,
 * cpGearJoint.c:91-102, cpSimpleMotor.c:87-96) */
static cpFloat default_spring_force_(cpConstraint *c, cpFloat dist) { return (c->restLength - dist)*c->stiffness; }
static cpFloat default_spring_torque_(cpConstraint *c, cpFloat relativeAngle) { return (relativeAngle - c->restAngle)*c->stiffness; }

cpConstraint *cpGrooveJointNew(cpBody *a, cpBody *b, cpVect groove_a, cpVect groove_b, cpVect anchorB)
{
	cpConstraint *c = cons_new_(CPG_GROOVE, a, b);
	c->grv_a = groove_a; c->grv_b = groove_b;
	c->grv_n = cpvperp(cpvnormalize(cpvsub(groove_b, groove_a)));
	c->anchorB = anchorB;
	return c;
}
cpConstraint *cpDampedSpringNew(cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB, cpFloat restLength, cpFloat stiffness, cpFloat damping)
{
	cpConstraint *c = cons_new_(CPG_DSPRING, a, b);
	c->anchorA = anchorA; c->anchorB = anchorB;
	c->restLength = restLength; c->stiffness = stiffness; c->damping = damping;
	c->springForceFunc = (cpDampedSpringForceFunc)default_spring_force_;
	return c;
}
cpConstraint *cpDampedRotarySpringNew(cpBody *a, cpBody *b, cpFloat restAngle, cpFloat stiffness, cpFloat damping)
{
	cpConstraint *c = cons_new_(CPG_DRSPRING, a, b);
	c->restAngle = restAngle; c->stiffness = stiffness; c->damping = damping;
	c->springTorqueFunc = (cpDampedRotarySpringTorqueFunc)default_spring_torque_;
	return c;
}
cpConstraint *cpRotaryLimitJointNew(cpBody *a, cpBody *b, cpFloat min, cpFloat max)
{
	cpConstraint *c = cons_new_(CPG_ROTLIMIT, a, b);
	c->min = min; c->max = max;
	return c;
}
cpConstraint *cpRatchetJointNew(cpBody *a, cpBody *b, cpFloat phase, cpFloat ratchet)
{
	cpConstraint *c = cons_new_(CPG_RATCHET, a, b);
	c->phase = phase; c->ratchet = ratchet;
	c->rec.angle = (b ? rd(b)->a : 0.0) - (a ? rd(a)->a : 0.0);
	return c;
}
cpConstraint *cpGearJointNew(cpBody *a, cpBody *b, cpFloat phase, cpFloat ratio)
{
	cpConstraint *c = cons_new_(CPG_GEAR, a, b);
	c->phase = phase; c->ratio = ratio; c->ratio_inv = 1.0/ratio;
	return c;
}
cpConstraint *cpSimpleMotorNew(cpBody *a, cpBody *b, cpFloat rate)
{
	cpConstraint *c = cons_new_(CPG_MOTOR, a, b);
	c->rate = rate;
	return c;
}

#define KIND_CHECK(c, k, what) ASSERT_HARD((c)->kind == (k), "Constraint is not a " what ".")
cpBool cpConstraintIsGrooveJoint(const cpConstraint *c) { return c->kind == CPG_GROOVE; }
cpBool cpConstraintIsDampedSpring(const cpConstraint *c) { return c->kind == CPG_DSPRING; }
cpBool cpConstraintIsDampedRotarySpring(const cpConstraint *c) { return c->kind == CPG_DRSPRING; }
cpBool cpConstraintIsRotaryLimitJoint(const cpConstraint *c) { return c->kind == CPG_ROTLIMIT; }
cpBool cpConstraintIsRatchetJoint(const cpConstraint *c) { return c->kind == CPG_RATCHET; }
cpBool cpConstraintIsGearJoint(const cpConstraint *c) { return c->kind == CPG_GEAR; }
cpBool cpConstraintIsSimpleMotor(const cpConstraint *c) { return c->kind == CPG_MOTOR; }
cpVect cpGrooveJointGetGrooveA(const cpConstraint *c) { KIND_CHECK(c, CPG_GROOVE, "groove joint"); return c->grv_a; }
void cpGrooveJointSetGrooveA(cpConstraint *c, cpVect v)
{
	KIND_CHECK(c, CPG_GROOVE, "groove joint");
	cwr(c)->grv_a = v; c->grv_n = cpvperp(cpvnormalize(cpvsub(c->grv_b, v)));
}
cpVect cpGrooveJointGetGrooveB(const cpConstraint *c) { KIND_CHECK(c, CPG_GROOVE, "groove joint"); return c->grv_b; }
void cpGrooveJointSetGrooveB(cpConstraint *c, cpVect v)
{
	KIND_CHECK(c, CPG_GROOVE, "groove joint");
	cwr(c)->grv_b = v; c->grv_n = cpvperp(cpvnormalize(cpvsub(v, c->grv_a)));
}
cpVect cpGrooveJointGetAnchorB(const cpConstraint *c) { KIND_CHECK(c, CPG_GROOVE, "groove joint"); return c->anchorB; }
void cpGrooveJointSetAnchorB(cpConstraint *c, cpVect v) { KIND_CHECK(c, CPG_GROOVE, "groove joint"); cwr(c)->anchorB = v; }
cpVect cpDampedSpringGetAnchorA(const cpConstraint *c) { KIND_CHECK(c, CPG_DSPRING, "damped spring"); return c->anchorA; }
void cpDampedSpringSetAnchorA(cpConstraint *c, cpVect v) { KIND_CHECK(c, CPG_DSPRING, "damped spring"); cwr(c)->anchorA = v; }
cpVect cpDampedSpringGetAnchorB(const cpConstraint *c) { KIND_CHECK(c, CPG_DSPRING, "damped spring"); return c->anchorB; }
void cpDampedSpringSetAnchorB(cpConstraint *c, cpVect v) { KIND_CHECK(c, CPG_DSPRING, "damped spring"); cwr(c)->anchorB = v; }
cpFloat cpDampedSpringGetRestLength(const cpConstraint *c) { KIND_CHECK(c, CPG_DSPRING, "damped spring"); return c->restLength; }
void cpDampedSpringSetRestLength(cpConstraint *c, cpFloat v) { KIND_CHECK(c, CPG_DSPRING, "damped spring"); cwr(c)->restLength = v; }
cpFloat cpDampedSpringGetStiffness(const cpConstraint *c) { KIND_CHECK(c, CPG_DSPRING, "damped spring"); return c->stiffness; }
void cpDampedSpringSetStiffness(cpConstraint *c, cpFloat v) { KIND_CHECK(c, CPG_DSPRING, "damped spring"); cwr(c)->stiffness = v; }
cpFloat cpDampedSpringGetDamping(const cpConstraint *c) { KIND_CHECK(c, CPG_DSPRING, "damped spring"); return c->damping; }
void cpDampedSpringSetDamping(cpConstraint *c, cpFloat v) { KIND_CHECK(c, CPG_DSPRING, "damped spring"); cwr(c)->damping = v; }
cpDampedSpringForceFunc cpDampedSpringGetSpringForceFunc(const cpConstraint *c) { KIND_CHECK(c, CPG_DSPRING, "damped spring"); return c->springForceFunc; }
void cpDampedSpringSetSpringForceFunc(cpConstraint *c, cpDampedSpringForceFunc f) { KIND_CHECK(c, CPG_DSPRING, "damped spring"); cwr(c)->springForceFunc = f; }
cpFloat cpDampedRotarySpringGetRestAngle(const cpConstraint *c) { KIND_CHECK(c, CPG_DRSPRING, "damped rotary spring"); return c->restAngle; }
void cpDampedRotarySpringSetRestAngle(cpConstraint *c, cpFloat v) { KIND_CHECK(c, CPG_DRSPRING, "damped rotary spring"); cwr(c)->restAngle = v; }
cpFloat cpDampedRotarySpringGetStiffness(const cpConstraint *c) { KIND_CHECK(c, CPG_DRSPRING, "damped rotary spring"); return c->stiffness; }
void cpDampedRotarySpringSetStiffness(cpConstraint *c, cpFloat v) { KIND_CHECK(c, CPG_DRSPRING, "damped rotary spring"); cwr(c)->stiffness = v; }
cpFloat cpDampedRotarySpringGetDamping(const cpConstraint *c) { KIND_CHECK(c, CPG_DRSPRING, "damped rotary spring"); return c->damping; }
void cpDampedRotarySpringSetDamping(cpConstraint *c, cpFloat v) { KIND_CHECK(c, CPG_DRSPRING, "damped rotary spring"); cwr(c)->damping = v; }
cpDampedRotarySpringTorqueFunc cpDampedRotarySpringGetSpringTorqueFunc(const cpConstraint *c) { KIND_CHECK(c, CPG_DRSPRING, "damped rotary spring"); return c->springTorqueFunc; }
void cpDampedRotarySpringSetSpringTorqueFunc(cpConstraint *c, cpDampedRotarySpringTorqueFunc f) { KIND_CHECK(c, CPG_DRSPRING, "damped rotary spring"); cwr(c)->springTorqueFunc = f; }
cpFloat cpRotaryLimitJointGetMin(const cpConstraint *c) { KIND_CHECK(c, CPG_ROTLIMIT, "rotary limit joint"); return c->min; }
void cpRotaryLimitJointSetMin(cpConstraint *c, cpFloat v) { KIND_CHECK(c, CPG_ROTLIMIT, "rotary limit joint"); cwr(c)->min = v; }
cpFloat cpRotaryLimitJointGetMax(const cpConstraint *c) { KIND_CHECK(c, CPG_ROTLIMIT, "rotary limit joint"); return c->max; }
void cpRotaryLimitJointSetMax(cpConstraint *c, cpFloat v) { KIND_CHECK(c, CPG_ROTLIMIT, "rotary limit joint"); cwr(c)->max = v; }
cpFloat cpRatchetJointGetAngle(const cpConstraint *c) { KIND_CHECK(c, CPG_RATCHET, "ratchet joint"); cons_pull_((cpConstraint *)c); return c->rec.angle; }
void cpRatchetJointSetAngle(cpConstraint *c, cpFloat v) { KIND_CHECK(c, CPG_RATCHET, "ratchet joint"); cwr(c)->rec.angle = v; }
cpFloat cpRatchetJointGetPhase(const cpConstraint *c) { KIND_CHECK(c, CPG_RATCHET, "ratchet joint"); return c->phase; }
void cpRatchetJointSetPhase(cpConstraint *c, cpFloat v) { KIND_CHECK(c, CPG_RATCHET, "ratchet joint"); cwr(c)->phase = v; }
cpFloat cpRatchetJointGetRatchet(const cpConstraint *c) { KIND_CHECK(c, CPG_RATCHET, "ratchet joint"); return c->ratchet; }
void cpRatchetJointSetRatchet(cpConstraint *c, cpFloat v) { KIND_CHECK(c, CPG_RATCHET, "ratchet joint"); cwr(c)->ratchet = v; }
cpFloat cpGearJointGetPhase(const cpConstraint *c) { KIND_CHECK(c, CPG_GEAR, "gear joint"); return c->phase; }
void cpGearJointSetPhase(cpConstraint *c, cpFloat v) { KIND_CHECK(c, CPG_GEAR, "gear joint"); cwr(c)->phase = v; }
cpFloat cpGearJointGetRatio(const cpConstraint *c) { KIND_CHECK(c, CPG_GEAR, "gear joint"); return c->ratio; }
void cpGearJointSetRatio(cpConstraint *c, cpFloat v) { KIND_CHECK(c, CPG_GEAR, "gear joint"); cwr(c)->ratio = v; c->ratio_inv = 1.0/v; }
cpFloat cpSimpleMotorGetRate(const cpConstraint *c) { KIND_CHECK(c, CPG_MOTOR, "simple motor"); return c->rate; }
void cpSimpleMotorSetRate(cpConstraint *c, cpFloat v) { KIND_CHECK(c, CPG_MOTOR, "simple motor"); cwr(c)->rate = v; }

/* ====================================================================
 * Space
 * ==================================================================== */
cpSpace *cpSpaceNew(void)
{
	/* cpSpace.c:119-178 (float literals: slop (double)0.1f, bias base 1.0f-0.1f) */
	cpSpace *sp = (cpSpace *)calloc(1, sizeof(cpSpace));
	sp->iterations = 10;
	sp->damping = 1.0;
	sp->collisionSlop = (cpFloat)0.1f;
	sp->collisionBias = pow((cpFloat)(1.0f - 0.1f), 60.0);
	sp->collisionPersistence = 3;
	sp->sleepTimeThreshold = INF_;
	memcpy(&sp->defaultHandler, &handler_do_nothing_, sizeof(cpCollisionHandler));
	sp->mode = CP_GPU_SOLVER_ORDERED;
	body_init_(&sp->staticBody, 0.0, 0.0);
	make_static_(&sp->staticBody);
	sp->staticBody.space = sp;
	return sp;
}

void cpSpaceDestroy(cpSpace *sp)
{
	if(!sp) return;
	if(sp->dev && sp->ownsDev){
		/* the bodies outlive the space: they keep its last step's state */
		space_pull(sp);
		cudaStreamSynchronize(lib_stream());
		devset_free(sp->dev);
	}
	/* cpSpace.c:186-191: every body is woken; here the sleeping ones are
	 * only let go of their components */
	for(int i = 0; i < sp->nslp; i++){
		cpBody *b = sp->slp[i];
		b->sleepRoot = b->sleepNext = NULL;
		b->idleTime = 0.0;
		if(b->space == sp) b->space = NULL;
	}
	graph_stop_(sp);
	free(sp->slp); free(sp->sleeping); free(sp->roused); free(sp->garb); free(sp->gfree); free(sp->glist);
	free(sp->sedKey); free(sp->sedOp); free(sp->sedStamp);
	sp->slp = sp->sleeping = sp->roused = NULL; sp->garb = NULL; sp->gfree = sp->glist = NULL;
	sp->sedKey = NULL; sp->sedOp = NULL; sp->sedStamp = NULL;
	sp->nslp = sp->nsleeping = sp->nroused = 0;
	for(int i = 0; i < sp->nhandlers; i++) free(sp->handlers[i]);
	free(sp->handlers); free(sp->harb); free(sp->udKey); free(sp->udVal);
	sp->handlers = NULL; sp->harb = NULL; sp->udKey = NULL; sp->udVal = NULL;
	sp->nhandlers = sp->caphandlers = sp->capharb = sp->udCap = sp->udUsed = 0;
	for(int i = 0; i < sp->ndyn; i++) if(sp->dyn[i]->space == sp) sp->dyn[i]->space = NULL;
	for(int i = 0; i < sp->nstat; i++) if(sp->stat[i]->space == sp) sp->stat[i]->space = NULL;
	for(int i = 0; i < sp->nshapes; i++) if(sp->shapes[i] && sp->shapes[i]->space == sp) sp->shapes[i]->space = NULL;
	for(int i = 0; i < sp->ncons; i++) if(sp->cons[i]->space == sp) sp->cons[i]->space = NULL;
	free(sp->dyn); free(sp->stat); free(sp->shapes); free(sp->cons); free(sp->ops); free(sp->snap); free(sp->post);
	sp->dyn = NULL; sp->stat = NULL; sp->shapes = NULL; sp->cons = NULL; sp->ops = NULL; sp->snap = NULL; sp->post = NULL;
	sp->dev = NULL;
}

void cpSpaceFree(cpSpace *sp)
{
	if(!sp) return;
	cpSpaceDestroy(sp);
	free(sp);
}

/* ---- caller-placed objects: the New functions' objects moved into the
 * caller's memory (no object refers to its own address except a space's
 * static body, re-pointed here) ---- */
static void *adopt_(void *mem, void *fresh, size_t bytes)
{
	if(mem && fresh) memcpy(mem, fresh, bytes);
	free(fresh);
	return mem;
}

cpSpace *cpSpaceAlloc(void) { return (cpSpace *)calloc(1, sizeof(cpSpace)); }
cpSpace *cpSpaceInit(cpSpace *sp)
{
	adopt_(sp, cpSpaceNew(), sizeof(cpSpace));
	sp->staticBody.space = sp;
	return sp;
}
cpBody *cpBodyAlloc(void) { return (cpBody *)calloc(1, sizeof(cpBody)); }
cpBody *cpBodyInit(cpBody *b, cpFloat mass, cpFloat moment) { return (cpBody *)adopt_(b, cpBodyNew(mass, moment), sizeof(cpBody)); }
void cpBodyDestroy(cpBody *b) { (void)b; }
void cpShapeDestroy(cpShape *s) { if(s){ free(s->lv); s->lv = s->ln = s->gv = s->gn = NULL; } }
void cpConstraintDestroy(cpConstraint *c) { (void)c; }

#define CPG_SHAPE_ALLOC(T) T *T##Alloc(void) { return (T *)calloc(1, sizeof(cpShape)); }
#define CPG_JOINT_ALLOC(T) T *T##Alloc(void) { return (T *)calloc(1, sizeof(cpConstraint)); }
CPG_SHAPE_ALLOC(cpCircleShape)
CPG_SHAPE_ALLOC(cpSegmentShape)
CPG_SHAPE_ALLOC(cpPolyShape)
CPG_JOINT_ALLOC(cpPivotJoint)
CPG_JOINT_ALLOC(cpPinJoint)
CPG_JOINT_ALLOC(cpSlideJoint)
CPG_JOINT_ALLOC(cpGrooveJoint)
CPG_JOINT_ALLOC(cpDampedSpring)
CPG_JOINT_ALLOC(cpDampedRotarySpring)
CPG_JOINT_ALLOC(cpRotaryLimitJoint)
CPG_JOINT_ALLOC(cpRatchetJoint)
CPG_JOINT_ALLOC(cpGearJoint)
CPG_JOINT_ALLOC(cpSimpleMotor)

cpCircleShape *cpCircleShapeInit(cpCircleShape *m, cpBody *body, cpFloat radius, cpVect offset)
{ return (cpCircleShape *)adopt_(m, cpCircleShapeNew(body, radius, offset), sizeof(cpShape)); }
cpSegmentShape *cpSegmentShapeInit(cpSegmentShape *m, cpBody *body, cpVect a, cpVect b, cpFloat radius)
{ return (cpSegmentShape *)adopt_(m, cpSegmentShapeNew(body, a, b, radius), sizeof(cpShape)); }
cpPolyShape *cpPolyShapeInit(cpPolyShape *m, cpBody *body, int count, const cpVect *verts, cpTransform transform, cpFloat radius)
{ return (cpPolyShape *)adopt_(m, cpPolyShapeNew(body, count, verts, transform, radius), sizeof(cpShape)); }
cpPolyShape *cpPolyShapeInitRaw(cpPolyShape *m, cpBody *body, int count, const cpVect *verts, cpFloat radius)
{ return (cpPolyShape *)adopt_(m, cpPolyShapeNewRaw(body, count, verts, radius), sizeof(cpShape)); }
cpPolyShape *cpBoxShapeInit(cpPolyShape *m, cpBody *body, cpFloat width, cpFloat height, cpFloat radius)
{ return (cpPolyShape *)adopt_(m, cpBoxShapeNew(body, width, height, radius), sizeof(cpShape)); }
cpPolyShape *cpBoxShapeInit2(cpPolyShape *m, cpBody *body, cpBB box, cpFloat radius)
{ return (cpPolyShape *)adopt_(m, cpBoxShapeNew2(body, box, radius), sizeof(cpShape)); }

cpPivotJoint *cpPivotJointInit(cpPivotJoint *m, cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB)
{ return (cpPivotJoint *)adopt_(m, cpPivotJointNew2(a, b, anchorA, anchorB), sizeof(cpConstraint)); }
cpPinJoint *cpPinJointInit(cpPinJoint *m, cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB)
{ return (cpPinJoint *)adopt_(m, cpPinJointNew(a, b, anchorA, anchorB), sizeof(cpConstraint)); }
cpSlideJoint *cpSlideJointInit(cpSlideJoint *m, cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB, cpFloat min, cpFloat max)
{ return (cpSlideJoint *)adopt_(m, cpSlideJointNew(a, b, anchorA, anchorB, min, max), sizeof(cpConstraint)); }
cpGrooveJoint *cpGrooveJointInit(cpGrooveJoint *m, cpBody *a, cpBody *b, cpVect groove_a, cpVect groove_b, cpVect anchorB)
{ return (cpGrooveJoint *)adopt_(m, cpGrooveJointNew(a, b, groove_a, groove_b, anchorB), sizeof(cpConstraint)); }
cpDampedSpring *cpDampedSpringInit(cpDampedSpring *m, cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB,
                                   cpFloat restLength, cpFloat stiffness, cpFloat damping)
{ return (cpDampedSpring *)adopt_(m, cpDampedSpringNew(a, b, anchorA, anchorB, restLength, stiffness, damping), sizeof(cpConstraint)); }
cpDampedRotarySpring *cpDampedRotarySpringInit(cpDampedRotarySpring *m, cpBody *a, cpBody *b, cpFloat restAngle,
                                               cpFloat stiffness, cpFloat damping)
{ return (cpDampedRotarySpring *)adopt_(m, cpDampedRotarySpringNew(a, b, restAngle, stiffness, damping), sizeof(cpConstraint)); }
cpRotaryLimitJoint *cpRotaryLimitJointInit(cpRotaryLimitJoint *m, cpBody *a, cpBody *b, cpFloat min, cpFloat max)
{ return (cpRotaryLimitJoint *)adopt_(m, cpRotaryLimitJointNew(a, b, min, max), sizeof(cpConstraint)); }
cpRatchetJoint *cpRatchetJointInit(cpRatchetJoint *m, cpBody *a, cpBody *b, cpFloat phase, cpFloat ratchet)
{ return (cpRatchetJoint *)adopt_(m, cpRatchetJointNew(a, b, phase, ratchet), sizeof(cpConstraint)); }
cpGearJoint *cpGearJointInit(cpGearJoint *m, cpBody *a, cpBody *b, cpFloat phase, cpFloat ratio)
{ return (cpGearJoint *)adopt_(m, cpGearJointNew(a, b, phase, ratio), sizeof(cpConstraint)); }
cpSimpleMotor *cpSimpleMotorInit(cpSimpleMotor *m, cpBody *a, cpBody *b, cpFloat rate)
{ return (cpSimpleMotor *)adopt_(m, cpSimpleMotorNew(a, b, rate), sizeof(cpConstraint)); }

/* cpHastySpace.c:453-548: the threaded space, here a space (the device
 * runs the solver); the thread count is stored and reported */
cpSpace *cpHastySpaceNew(void) { return cpSpaceNew(); }
void cpHastySpaceFree(cpSpace *sp) { cpSpaceFree(sp); }
void cpHastySpaceSetThreads(cpSpace *sp, unsigned long threads) { if(sp) sp->hastyThreads = threads; }
unsigned long cpHastySpaceGetThreads(cpSpace *sp) { return (sp && sp->hastyThreads) ? sp->hastyThreads : 1ul; }
void cpHastySpaceStep(cpSpace *sp, cpFloat dt) { cpSpaceStep(sp, dt); }

int cpSpaceGetIterations(const cpSpace *sp) { return sp->iterations; }
void cpSpaceSetIterations(cpSpace *sp, int it) { ASSERT_HARD(it > 0, "Iterations must be positive and non-zero."); sp->iterations = it; }
cpVect cpSpaceGetGravity(const cpSpace *sp) { return sp->gravity; }
/* cpSpace.c:253-263: the sleeping components are woken as the reference
 * wakes them, walking the array that each activation shrinks */
void cpSpaceSetGravity(cpSpace *sp, cpVect g)
{
	sp->gravity = g;
	for(int i = 0; i < sp->nsleeping; i++) cpBodyActivate(sp->sleeping[i]);
}
cpFloat cpSpaceGetDamping(const cpSpace *sp) { return sp->damping; }
void cpSpaceSetDamping(cpSpace *sp, cpFloat d) { ASSERT_HARD(d >= 0.0, "Damping must be positive."); sp->damping = d; }
cpFloat cpSpaceGetIdleSpeedThreshold(const cpSpace *sp) { return sp->idleSpeedThreshold; }
void cpSpaceSetIdleSpeedThreshold(cpSpace *sp, cpFloat v) { sp->idleSpeedThreshold = v; }
cpFloat cpSpaceGetSleepTimeThreshold(const cpSpace *sp) { return sp->sleepTimeThreshold; }
void cpSpaceSetSleepTimeThreshold(cpSpace *sp, cpFloat t)
{
	sp->sleepTimeThreshold = t;
	/* the contact graph is kept from now on */
	if(t != INF_) graph_start_(sp);
}
cpFloat cpSpaceGetCollisionSlop(const cpSpace *sp) { return sp->collisionSlop; }
void cpSpaceSetCollisionSlop(cpSpace *sp, cpFloat v) { sp->collisionSlop = v; }
cpFloat cpSpaceGetCollisionBias(const cpSpace *sp) { return sp->collisionBias; }
void cpSpaceSetCollisionBias(cpSpace *sp, cpFloat v) { sp->collisionBias = v; }
cpTimestamp cpSpaceGetCollisionPersistence(const cpSpace *sp) { return sp->collisionPersistence; }
void cpSpaceSetCollisionPersistence(cpSpace *sp, cpTimestamp v) { sp->collisionPersistence = v; }
cpDataPointer cpSpaceGetUserData(const cpSpace *sp) { return sp->userData; }
void cpSpaceSetUserData(cpSpace *sp, cpDataPointer d) { sp->userData = d; }
cpBody *cpSpaceGetStaticBody(const cpSpace *sp) { return (cpBody *)&sp->staticBody; }
cpFloat cpSpaceGetCurrentTimeStep(const cpSpace *sp) { return sp->curr_dt; }
/* locked while queries, iterations and the step's callbacks run */
cpBool cpSpaceIsLocked(cpSpace *sp) { return sp->locked > 0; }
cpBool cpSpaceContainsShape(cpSpace *sp, cpShape *s) { return s->space == sp; }
cpBool cpSpaceContainsBody(cpSpace *sp, cpBody *b) { return b->space == sp; }
cpBool cpSpaceContainsConstraint(cpSpace *sp, cpConstraint *c) { return c->space == sp; }
void cpGpuSetSolverMode(cpSpace *sp, int mode)
{
	if(mode < CP_GPU_SOLVER_ORDERED || mode > CP_GPU_SOLVER_COLORED){
		set_error(CP_GPU_ERR_ARGUMENT, "unknown solver mode %d", mode);
		return;
	}
	sp->mode = mode;
}
int cpGpuGetSolverMode(const cpSpace *sp) { return sp->mode; }

/* Objects are about to be added or removed while the space's state is on
 * the device: bring it home (bodies, joint accumulators, shape boxes), so
 * the host holds the whole state until the next step rebuilds the set. */
static void space_detach(cpSpace *sp)
{
	if(!sp || !sp->dev || sp->structDirty || !sp->ownsDev) return;
	space_pull(sp);
	joints_pull_(sp);
	shapes_pull_all_(sp);
	sp->structDirty = 1;
	sp->snapValid = 0;
}

/* Whether the space's objects may change now.  A space stepped in a batch
 * keeps the objects it joined with. */
static int space_edit_ok(cpSpace *sp)
{
	if(sp->dev && !sp->ownsDev){
		set_error(CP_GPU_ERR_UNSUPPORTED, "a space stepped in a cpGpuBatch cannot gain or lose objects");
		return 0;
	}
	space_detach(sp);
	return 1;
}

/* cpArrayDeleteObj (cpArray.c:76-88): the last element takes the hole. */
static int array_delete_(void **arr, int *n, void *obj)
{
	for(int i = 0; i < *n; i++){
		if(arr[i] == obj){
			(*n)--;
			arr[i] = arr[*n];
			arr[*n] = NULL;
			return i;
		}
	}
	return -1;
}

static void record_op_(cpSpace *sp, int kind, cpShape *s, int isStatic)
{
	if(sp->nops == sp->capops){
		sp->capops = sp->capops ? 2*sp->capops : 256;
		sp->ops = (cpgOp *)realloc(sp->ops, sizeof(cpgOp)*(size_t)sp->capops);
	}
	cpgOp *op = &sp->ops[sp->nops++];
	memset(op, 0, sizeof(*op));
	op->shape = (int)s->hashid;
	op->isStatic = isStatic;
	op->kind = kind;
	if(kind == CPG_OP_INSERT || kind == CPG_OP_REINDEX){
		/* the box as cached now and the body's velocity now: the leaf's
		 * fattened box is made at this call (cpBBTree.c:82-98, 605-616) */
		op->l = s->bb.l; op->b = s->bb.b; op->r = s->bb.r; op->t = s->bb.t;
		op->vx = s->body->v.x; op->vy = s->body->v.y;
	}
}

/* ====================================================================
 * Sleeping and the contact graph (src/cpSpaceComponent.c)
 *
 * While sleeping is on (a finite sleep time threshold, or bodies still
 * asleep) a step stops once its arbiter list is built.  The host reads
 * the list and the bodies, rebuilds the contact graph and runs
 * cpSpaceProcessComponents on its own objects: idle times, bodies woken
 * by contacts, components put to sleep.  A step where no body wakes or
 * falls asleep goes straight on to the solve.  A step where some do edits
 * the host's arrays as the reference does (the dynamic and constraint
 * arrays, the arbiter list, the shapes' indices), rebuilds the device set
 * with the index edits replayed, marks the arbiters that left or rejoined
 * the cache, writes the new arbiter list, and then solves.  A sleeping
 * body stays on the device past the dynamic array, so it is neither
 * integrated nor re-indexed; its shapes sit in the static index.
 * ==================================================================== */
static int sleep_mode_(const cpSpace *sp) { return sp->sleepTimeThreshold != INF_ || sp->nsleeping > 0; }

/* the device table's key of a shape pair (world 0) */
static inline unsigned long long garb_key_(int a, int b)
{
	unsigned long long lo = (unsigned long long)(a < b ? a : b), hi = (unsigned long long)(a < b ? b : a);
	return ((lo << 21) | hi) + 2ull;
}

#define GARB_AT_(sp, k) (&(sp)->garb[(k) - 1])   /* k: pool index + 1 */

static int garb_alloc_(cpSpace *sp)
{
	int g;
	if(sp->ngfree > 0) g = sp->gfree[--sp->ngfree];
	else {
		if(sp->ngarb == sp->capgarb){
			sp->capgarb = sp->capgarb ? 2*sp->capgarb : 256;
			sp->garb = (cpArbiter *)realloc(sp->garb, sizeof(cpArbiter)*(size_t)sp->capgarb);
		}
		g = sp->ngarb++;
	}
	memset(&sp->garb[g], 0, sizeof(cpArbiter));
	sp->garb[g].listPos = -1;
	return g;
}

static void garb_release_(cpSpace *sp, int g)
{
	if(sp->ngfree == sp->capgfree){
		sp->capgfree = sp->capgfree ? 2*sp->capgfree : 256;
		sp->gfree = (int *)realloc(sp->gfree, sizeof(int)*(size_t)sp->capgfree);
	}
	sp->garb[g].a = sp->garb[g].b = NULL;
	sp->gfree[sp->ngfree++] = g;
}

/* cpArbiterThreadForBody (chipmunk_private.h:178-181) */
static int *gprev_(cpArbiter *arb, const cpBody *body) { return (arb->body_a == body) ? &arb->prevA : &arb->prevB; }
static int *gnext_(cpArbiter *arb, const cpBody *body) { return (arb->body_a == body) ? &arb->nextA : &arb->nextB; }
static int garb_next_(cpSpace *sp, int k, const cpBody *body) { return *gnext_(GARB_AT_(sp, k), body); }

/* cpBodyPushArbiter (cpSpaceComponent.c:168-181) */
static void gpush_(cpSpace *sp, cpBody *body, int g)
{
	int next = body->arbList;
	*gnext_(&sp->garb[g], body) = next;
	if(next) *gprev_(GARB_AT_(sp, next), body) = g + 1;
	body->arbList = g + 1;
}

/* unthreadHelper / cpArbiterUnthread (cpArbiter.c:222-247) */
static void gunthread_body_(cpSpace *sp, int g, cpBody *body)
{
	cpArbiter *arb = &sp->garb[g];
	int prev = *gprev_(arb, body), next = *gnext_(arb, body);
	if(prev) *gnext_(GARB_AT_(sp, prev), body) = next;
	else if(body->arbList == g + 1) body->arbList = next;
	if(next) *gprev_(GARB_AT_(sp, next), body) = prev;
	*gprev_(arb, body) = 0;
	*gnext_(arb, body) = 0;
}

static void gunthread_(cpSpace *sp, int g)
{
	gunthread_body_(sp, g, sp->garb[g].body_a);
	gunthread_body_(sp, g, sp->garb[g].body_b);
}

static int gthreaded_(const cpSpace *sp, int g)
{
	const cpArbiter *arb = &sp->garb[g];
	return arb->prevA || arb->nextA || arb->prevB || arb->nextB ||
		arb->body_a->arbList == g + 1 || arb->body_b->arbList == g + 1;
}

static void glist_push_(cpSpace *sp, int g)
{
	if(sp->nglist == sp->capglist){
		sp->capglist = sp->capglist ? 2*sp->capglist : 256;
		sp->glist = (int *)realloc(sp->glist, sizeof(int)*(size_t)sp->capglist);
	}
	sp->garb[g].listPos = sp->nglist;
	sp->glist[sp->nglist++] = g;
}

/* cpArrayDeleteObj (cpArray.c:76-88) on the arbiter list */
static void glist_delete_(cpSpace *sp, int g)
{
	int i = sp->garb[g].listPos;
	if(i < 0) return;
	int last = sp->glist[--sp->nglist];
	sp->glist[i] = last;
	sp->garb[last].listPos = i;
	sp->garb[g].listPos = -1;
}

/* a device arbiter record into a graph entry (links kept) */
static void garb_fill_(cpSpace *sp, cpArbiter *arb, const cpgArb *g)
{
	arb->a = sp->shapes[g->a]; arb->b = sp->shapes[g->b];
	arb->body_a = arb->a->body; arb->body_b = arb->b->body;
	arb->count = g->count; arb->state = g->state;
	arb->n = cpv(g->nx, g->ny); arb->surface_vr = cpv(g->svx, g->svy);
	arb->e = g->e; arb->u = g->u; arb->swapped = cpFalse;
	arb->c[0] = g->c[0]; arb->c[1] = g->c[1];
	arb->key = garb_key_(g->a, g->b);
}

/* The device's arbiter list (n records), or NULL. */
static cpgArb *gather_list_(cpSpace *sp, int *count)
{
	DevSet *ds = sp->dev;
	cpgTree T;
	*count = 0;
	if(!d2h(&T, ds->d.tree + sp->world, sizeof(cpgTree)) || !cuda_ok(cudaStreamSynchronize(lib_stream()), "list")) return NULL;
	int n = T.narb;
	if(n > ds->gatherCap){
		if(ds->gather) cudaFree(ds->gather);
		ds->gatherCap = n + n/2 + 64;
		if(!cuda_ok(cudaMalloc((void **)&ds->gather, sizeof(cpgArb)*(size_t)ds->gatherCap), "gather")){ ds->gatherCap = 0; ds->gather = NULL; return NULL; }
	}
	cpgArb *host = HALLOC(cpgArb, n);
	if(n > 0){
		cpg_launch_gather_arbs(&ds->d, sp->world, ds->gather, n, lib_stream());
		d2h(host, ds->gather, sizeof(cpgArb)*(size_t)n);
		if(!cuda_ok(cudaStreamSynchronize(lib_stream()), "list")){ free(host); return NULL; }
	}
	*count = n;
	return host;
}

/* A graph entry's record fields from the device's record (links kept). */
static void graph_fill_keep_(cpSpace *sp, cpArbiter *arb, const cpgArb *g)
{
	unsigned long long key = arb->key;
	int pa = arb->prevA, na = arb->nextA, pb = arb->prevB, nb = arb->nextB, lp = arb->listPos;
	garb_fill_(sp, arb, g);
	arb->key = key; arb->prevA = pa; arb->nextA = na; arb->prevB = pb; arb->nextB = nb; arb->listPos = lp;
}

/* The graph entries brought to the device's records for cpBodyEachArbiter:
 * the list's (after a solve: accumulated impulses) and, by key, the ones
 * sleeping bodies hold. */
static void graph_refresh_(cpSpace *sp)
{
	if(sp->graphFresh || !sp->dev || sp->structDirty || !sp->ownsDev) return;
	int n = 0;
	cpgArb *recs = gather_list_(sp, &n);
	if(!recs) return;
	for(int i = 0; i < n && i < sp->nglist; i++) graph_fill_keep_(sp, &sp->garb[sp->glist[i]], &recs[i]);
	free(recs);
	int m = 0;
	int *idx = HALLOC(int, sp->ngarb);
	unsigned long long *keys = HALLOC(unsigned long long, sp->ngarb);
	for(int g = 0; g < sp->ngarb; g++){
		if(sp->garb[g].a && sp->garb[g].listPos < 0){ idx[m] = g; keys[m] = sp->garb[g].key; m++; }
	}
	DevSet *ds = sp->dev;
	if(m > 0 && m <= ds->gatherCap){
		size_t kb = sizeof(unsigned long long)*(size_t)m;
		if(ds->qbytes < kb){
			if(ds->qbuf) cudaFree(ds->qbuf);
			ds->qbuf = NULL; ds->qbytes = 0;
			if(cuda_ok(cudaMalloc(&ds->qbuf, kb), "cudaMalloc graph keys")) ds->qbytes = kb;
		}
		cpgArb *out = HALLOC(cpgArb, m);
		if(ds->qbytes >= kb && h2d(ds->qbuf, keys, kb) &&
		   cpg_launch_gather_keys(&ds->d, (const unsigned long long *)ds->qbuf, ds->gather, m, lib_stream()) == 0 &&
		   d2h(out, ds->gather, sizeof(cpgArb)*(size_t)m) && cuda_ok(cudaStreamSynchronize(lib_stream()), "graph records")){
			for(int i = 0; i < m; i++) if(out[i].a >= 0) graph_fill_keep_(sp, &sp->garb[idx[i]], &out[i]);
		}
		free(out);
	}
	free(idx); free(keys);
	sp->graphFresh = 1;
}

/* The shape pairs of the device's arbiter list, 2 ints each, or NULL. */
static int *gather_pairs_(cpSpace *sp, int *count)
{
	DevSet *ds = sp->dev;
	cpgTree T;
	*count = 0;
	if(!d2h(&T, ds->d.tree + sp->world, sizeof(cpgTree)) || !cuda_ok(cudaStreamSynchronize(lib_stream()), "list")) return NULL;
	int n = T.narb;
	if(n > ds->gatherCap){
		if(ds->gather) cudaFree(ds->gather);
		ds->gatherCap = n + n/2 + 64;
		if(!cuda_ok(cudaMalloc((void **)&ds->gather, sizeof(cpgArb)*(size_t)ds->gatherCap), "gather")){ ds->gatherCap = 0; ds->gather = NULL; return NULL; }
	}
	int *host = HALLOC(int, 2*n);
	if(n > 0){
		cpg_launch_gather_pairs(&ds->d, sp->world, (int *)ds->gather, n, lib_stream());
		d2h(host, ds->gather, sizeof(int)*2*(size_t)n);
		if(!cuda_ok(cudaStreamSynchronize(lib_stream()), "list pairs")){ free(host); return NULL; }
	}
	*count = n;
	return host;
}

/* The graph starts from the last step's list, threaded in list order as
 * cpSpaceProcessComponents threads it on every step. */
static void graph_start_(cpSpace *sp)
{
	if(sp->graphOn) return;
	sp->graphOn = 1;
	sp->graphFresh = 1;
	if(!sp->dev || !sp->ownsDev) return;
	int n = 0;
	cpgArb *recs = gather_list_(sp, &n);
	if(!recs) return;
	for(int i = 0; i < n; i++){
		const cpgArb *r = &recs[i];
		if(r->a < 0 || r->a >= sp->nshapes || r->b < 0 || r->b >= sp->nshapes || !sp->shapes[r->a] || !sp->shapes[r->b]) continue;
		int g = garb_alloc_(sp);
		garb_fill_(sp, &sp->garb[g], r);
		glist_push_(sp, g);
		gpush_(sp, sp->garb[g].body_a, g);
		gpush_(sp, sp->garb[g].body_b, g);
	}
	free(recs);
}

static void graph_stop_(cpSpace *sp)
{
	if(!sp->graphOn) return;
	for(int g = 0; g < sp->ngarb; g++){
		cpArbiter *arb = &sp->garb[g];
		if(arb->a){ arb->body_a->arbList = 0; arb->body_b->arbList = 0; }
	}
	sp->ngarb = sp->ngfree = sp->nglist = sp->nsed = 0;
	sp->graphOn = 0;
}

static void sed_push_(cpSpace *sp, unsigned long long key, int op)
{
	if(sp->nsed == sp->capsed){
		sp->capsed = sp->capsed ? 2*sp->capsed : 64;
		sp->sedKey = (unsigned long long *)realloc(sp->sedKey, sizeof(unsigned long long)*(size_t)sp->capsed);
		sp->sedOp = (int *)realloc(sp->sedOp, sizeof(int)*(size_t)sp->capsed);
		sp->sedStamp = (unsigned *)realloc(sp->sedStamp, sizeof(unsigned)*(size_t)sp->capsed);
	}
	sp->sedKey[sp->nsed] = key; sp->sedOp[sp->nsed] = op; sp->sedStamp[sp->nsed] = (unsigned)sp->stamp;
	sp->nsed++;
}

/* After a rebuild: the cache edits in call order and the arbiter list. */
static int sleep_apply_edits_(cpSpace *sp)
{
	if(!sp->graphOn || !sp->dev) return 1;
	DevSet *ds = sp->dev;
	size_t kb = align256(sizeof(unsigned long long)*(size_t)(sp->nsed + 1));
	size_t ob = align256(sizeof(int)*(size_t)(sp->nsed + 1));
	size_t sb = align256(sizeof(unsigned)*(size_t)(sp->nsed + 1));
	size_t lb = align256(sizeof(unsigned long long)*(size_t)(sp->nglist + 1));
	size_t need = kb + ob + sb + lb;
	if(ds->qbytes < need){
		if(ds->qbuf) cudaFree(ds->qbuf);
		ds->qbuf = NULL; ds->qbytes = 0;
		if(!cuda_ok(cudaMalloc(&ds->qbuf, need), "cudaMalloc sleeping edits")) return 0;
		ds->qbytes = need;
	}
	char *base = (char *)ds->qbuf;
	unsigned long long *lkeys = HALLOC(unsigned long long, sp->nglist);
	for(int i = 0; i < sp->nglist; i++) lkeys[i] = sp->garb[sp->glist[i]].key;
	int ok = 1;
	if(sp->nsed > 0){
		ok &= h2d(base, sp->sedKey, sizeof(unsigned long long)*(size_t)sp->nsed);
		ok &= h2d(base + kb, sp->sedOp, sizeof(int)*(size_t)sp->nsed);
		ok &= h2d(base + kb + ob, sp->sedStamp, sizeof(unsigned)*(size_t)sp->nsed);
	}
	if(sp->nglist > 0) ok &= h2d(base + kb + ob + sb, lkeys, sizeof(unsigned long long)*(size_t)sp->nglist);
	ok &= cpg_launch_sleep_edits(&ds->d, (const unsigned long long *)base, (const int *)(base + kb), (const unsigned *)(base + kb + ob),
	                             sp->nsed, (const unsigned long long *)(base + kb + ob + sb), sp->nglist, lib_stream()) == 0;
	/* the pageable copies above must finish before lkeys goes */
	ok &= cuda_ok(cudaStreamSynchronize(lib_stream()), "sleeping edits");
	free(lkeys);
	sp->nsed = 0;
	return ok;
}

/* Before the first array edit of a wake or a sleep: the state comes home
 * (space_detach), so the next step or query rebuilds the set. */
static void sleep_mutate_(cpSpace *sp)
{
	space_detach(sp);
	if(sp->dev) sp->structDirty = 1;
	sp->sleepMutated = 1;
	sp->snapValid = 0;
}

static void space_unlock_(cpSpace *sp);

/* cpSpaceActivateBody (cpSpaceComponent.c:28-79) */
static void space_activate_body_(cpSpace *sp, cpBody *body)
{
	if(sp->locked){
		for(int i = 0; i < sp->nroused; i++) if(sp->roused[i] == body) return;
		push_((void ***)&sp->roused, &sp->nroused, &sp->caproused, body);
		return;
	}
	sleep_mutate_(sp);
	array_delete_((void **)sp->slp, &sp->nslp, body);
	push_((void ***)&sp->dyn, &sp->ndyn, &sp->capdyn, body);
	for(cpShape *s = body->shapeList; s; s = s->next){
		record_op_(sp, CPG_OP_REMOVE, s, 1);
		record_op_(sp, CPG_OP_INSERT, s, 0);
	}
	for(int k = body->arbList; k; k = garb_next_(sp, k, body)){
		cpArbiter *arb = GARB_AT_(sp, k);
		if(body == arb->body_a || body_type_(arb->body_a) == CP_BODY_TYPE_STATIC){
			sed_push_(sp, arb->key, 0);
			glist_push_(sp, k - 1);
		}
	}
	for(cpConstraint *c = body->constraintList; c; c = cons_next_(c, body)){
		if(body == c->a || body_type_(c->a) == CP_BODY_TYPE_STATIC){
			c->index = sp->ncons;
			push_((void ***)&sp->cons, &sp->ncons, &sp->capcons, c);
		}
	}
}

/* cpSpaceDeactivateBody (cpSpaceComponent.c:81-112) */
static void space_deactivate_body_(cpSpace *sp, cpBody *body)
{
	sleep_mutate_(sp);
	array_delete_((void **)sp->dyn, &sp->ndyn, body);
	push_((void ***)&sp->slp, &sp->nslp, &sp->capslp, body);
	for(cpShape *s = body->shapeList; s; s = s->next){
		record_op_(sp, CPG_OP_REMOVE, s, 0);
		record_op_(sp, CPG_OP_INSERT, s, 1);
	}
	for(int k = body->arbList; k; k = garb_next_(sp, k, body)){
		cpArbiter *arb = GARB_AT_(sp, k);
		if(body == arb->body_a || body_type_(arb->body_a) == CP_BODY_TYPE_STATIC){
			sed_push_(sp, arb->key, 1);
			glist_delete_(sp, k - 1);
		}
	}
	for(cpConstraint *c = body->constraintList; c; c = cons_next_(c, body)){
		if(body == c->a || body_type_(c->a) == CP_BODY_TYPE_STATIC){
			int i = array_delete_((void **)sp->cons, &sp->ncons, c);
			if(i >= 0 && i < sp->ncons) sp->cons[i]->index = i;
		}
	}
}

cpBool cpBodyIsSleeping(const cpBody *b) { return b->sleepRoot != NULL; }

/* cpSpaceComponent.c:120-153 */
void cpBodyActivate(cpBody *body)
{
	if(body == NULL || body_type_(body) != CP_BODY_TYPE_DYNAMIC) return;
	body->idleTime = 0.0;
	cpBody *root = body->sleepRoot;
	if(root && cpBodyIsSleeping(root)){
		cpSpace *sp = root->space;
		cpBody *b = root;
		while(b){
			cpBody *next = b->sleepNext;
			b->idleTime = 0.0;
			b->sleepRoot = NULL;
			b->sleepNext = NULL;
			space_activate_body_(sp, b);
			b = next;
		}
		array_delete_((void **)sp->sleeping, &sp->nsleeping, root);
	}
	cpSpace *sp = body->space;
	if(!sp || !sp->graphOn) return;
	for(int k = body->arbList; k; k = garb_next_(sp, k, body)){
		cpArbiter *arb = GARB_AT_(sp, k);
		cpBody *other = (arb->body_a == body ? arb->body_b : arb->body_a);
		if(body_type_(other) != CP_BODY_TYPE_STATIC) other->idleTime = 0.0;
	}
}

/* cpSpaceComponent.c:155-166 */
void cpBodyActivateStatic(cpBody *body, cpShape *filter)
{
	ASSERT_HARD(body_type_(body) == CP_BODY_TYPE_STATIC, "cpBodyActivateStatic() called on a non-static body.");
	cpSpace *sp = body->space;
	if(!sp || !sp->graphOn) return;
	for(int k = body->arbList; k; k = garb_next_(sp, k, body)){
		cpArbiter *arb = GARB_AT_(sp, k);
		if(!filter || filter == arb->a || filter == arb->b) cpBodyActivate(arb->body_a == body ? arb->body_b : arb->body_a);
	}
}

/* FloodFillComponent with ComponentAdd (cpSpaceComponent.c:183-212) */
static void flood_fill_(cpSpace *sp, cpBody *root, cpBody *body)
{
	if(body_type_(body) != CP_BODY_TYPE_DYNAMIC || body->sleepRoot != NULL) return;
	body->sleepRoot = root;
	if(body != root){
		body->sleepNext = root->sleepNext;
		root->sleepNext = body;
	}
	for(int k = body->arbList; k; k = garb_next_(sp, k, body)){
		cpArbiter *arb = GARB_AT_(sp, k);
		flood_fill_(sp, root, body == arb->body_a ? arb->body_b : arb->body_a);
	}
	for(cpConstraint *c = body->constraintList; c; c = cons_next_(c, body)) flood_fill_(sp, root, body == c->a ? c->b : c->a);
}

/* cpSpaceProcessComponents (cpSpaceComponent.c:224-307) on the host's
 * objects; the bodies hold the state of this step's position update. */
static void process_components_(cpSpace *sp, cpFloat dt)
{
	int sleep = (sp->sleepTimeThreshold != INF_);
	if(sleep){
		cpFloat dv = sp->idleSpeedThreshold;
		cpFloat dvsq = (dv ? dv*dv : cpvlengthsq(sp->gravity)*dt*dt);
		for(int i = 0; i < sp->ndyn; i++){
			cpBody *body = sp->dyn[i];
			if(body_type_(body) != CP_BODY_TYPE_DYNAMIC) continue;
			cpFloat keThreshold = (dvsq ? body->m*dvsq : 0.0);
			/* cpBodyKineticEnergy (cpBody.c:581-588) */
			cpFloat vsq = cpvdot(body->v, body->v), wsq = body->w*body->w;
			cpFloat ke = (vsq ? vsq*body->m : 0.0) + (wsq ? wsq*body->i : 0.0);
			body->idleTime = (ke > keThreshold ? 0.0 : body->idleTime + dt);
		}
	}
	for(int i = 0, count = sp->nglist; i < count; i++){
		int g = sp->glist[i];
		cpBody *a = sp->garb[g].body_a, *b = sp->garb[g].body_b;
		if(sleep){
			if(body_type_(b) == CP_BODY_TYPE_KINEMATIC || cpBodyIsSleeping(a)) cpBodyActivate(a);
			if(body_type_(a) == CP_BODY_TYPE_KINEMATIC || cpBodyIsSleeping(b)) cpBodyActivate(b);
		}
		gpush_(sp, a, g);
		gpush_(sp, b, g);
	}
	if(!sleep) return;
	for(int i = 0; i < sp->ncons; i++){
		cpBody *a = sp->cons[i]->a, *b = sp->cons[i]->b;
		if(body_type_(b) == CP_BODY_TYPE_KINEMATIC) cpBodyActivate(a);
		if(body_type_(a) == CP_BODY_TYPE_KINEMATIC) cpBodyActivate(b);
	}
	for(int i = 0; i < sp->ndyn;){
		cpBody *body = sp->dyn[i];
		if(body->sleepRoot == NULL){
			flood_fill_(sp, body, body);
			/* ComponentActive (cpSpaceComponent.c:214-222) */
			int active = 0;
			for(cpBody *o = body; o; o = o->sleepNext) if(o->idleTime < sp->sleepTimeThreshold){ active = 1; break; }
			if(!active){
				push_((void ***)&sp->sleeping, &sp->nsleeping, &sp->capsleeping, body);
				for(cpBody *o = body; o; o = o->sleepNext) space_deactivate_body_(sp, o);
				continue;
			}
		}
		i++;
		body->sleepRoot = NULL;
		body->sleepNext = NULL;
	}
}

/* The host half of a sleeping step, between the device's two halves:
 * cpSpaceStep.c:351-360 (the last list leaves the graph) and :375. */
static int sleep_sync_(cpSpace *sp, cpFloat dt)
{
	int n = 0;
	int *pairs = gather_pairs_(sp, &n);
	if(!pairs) return 0;
	space_pull(sp);
	for(int i = 0; i < sp->nglist; i++){
		int g = sp->glist[i];
		cpArbiter *arb = &sp->garb[g];
		arb->listPos = -1;
		if(!cpBodyIsSleeping(arb->body_a) && !cpBodyIsSleeping(arb->body_b)) gunthread_(sp, g);
	}
	for(int i = 0; i < sp->nglist; i++) if(!gthreaded_(sp, sp->glist[i])) garb_release_(sp, sp->glist[i]);
	sp->nglist = 0;
	for(int i = 0; i < n; i++){
		int g = garb_alloc_(sp);
		cpArbiter *arb = &sp->garb[g];
		/* the shapes and key now; the rest when cpBodyEachArbiter asks */
		arb->a = sp->shapes[pairs[2*i]]; arb->b = sp->shapes[pairs[2*i + 1]];
		arb->body_a = arb->a->body; arb->body_b = arb->b->body;
		arb->key = garb_key_(pairs[2*i], pairs[2*i + 1]);
		glist_push_(sp, g);
	}
	free(pairs);
	process_components_(sp, dt);
	sp->graphFresh = 0;
	if(sp->sleepMutated && !space_device_ready_(sp)) return 0;
	return 1;
}

/* cpSpaceUnlock (cpSpaceStep.c:68-103): bodies woken while the space was
 * locked are activated */
static void space_unlock_(cpSpace *sp)
{
	sp->locked--;
	if(sp->locked) return;
	for(int i = 0, count = sp->nroused; i < count; i++) space_activate_body_(sp, sp->roused[i]);
	sp->nroused = 0;
}

void cpBodySleep(cpBody *body) { cpBodySleepWithGroup(body, NULL); }

/* cpSpaceComponent.c:315-350 */
void cpBodySleepWithGroup(cpBody *body, cpBody *group)
{
	ASSERT_HARD(body_type_(body) == CP_BODY_TYPE_DYNAMIC, "Non-dynamic bodies cannot be put to sleep.");
	cpSpace *sp = body->space;
	ASSERT_HARD(!sp->locked, "Bodies cannot be put to sleep during a query or a call to cpSpaceStep(). Put these calls into a post-step callback.");
	ASSERT_HARD(sp->sleepTimeThreshold < INF_, "Sleeping is not enabled on the space. You cannot sleep a body without setting a sleep time threshold on the space.");
	ASSERT_HARD(group == NULL || cpBodyIsSleeping(group), "Cannot use a non-sleeping body as a group identifier.");
	if(cpBodyIsSleeping(body)){
		ASSERT_HARD(body->sleepRoot == (group ? group->sleepRoot : NULL), "The body is already sleeping and it's group cannot be reassigned.");
		return;
	}
	if(!space_edit_ok(sp)) return;
	for(cpShape *s = body->shapeList; s; s = s->next) cpShapeCacheBB(s);
	space_deactivate_body_(sp, body);
	if(group){
		cpBody *root = group->sleepRoot;
		body->sleepRoot = root;
		body->sleepNext = root->sleepNext;
		body->idleTime = 0.0;
		root->sleepNext = body;
	} else {
		body->sleepRoot = body;
		body->sleepNext = NULL;
		body->idleTime = 0.0;
		push_((void ***)&sp->sleeping, &sp->nsleeping, &sp->capsleeping, body);
	}
	/* cpSpaceComponent.c:349: a second delete, of a body no longer there */
	array_delete_((void **)sp->dyn, &sp->ndyn, body);
}

/* ====================================================================
 * Collision handlers (src/cpSpace.c:62-103, 378-413, src/cpArbiter.c)
 *
 * Once a handler is added, a step stops after the arbiter cache update:
 * every colliding arbiter is on the list in the reference's collision
 * order, with its sensor and ignore rule left to the host.  The host runs
 * begin and pre-solve on each (cpSpaceStep.c:259-283), applies the rule,
 * writes the changed records back and the list of the arbiters that stay.
 * The cache filter runs next on its own, and the host calls separate on
 * the arbiters it moved to the cached state; then the solve, and the host
 * calls post-solve on the list with the solved impulses.
 * ==================================================================== */
cpBool cpArbiterCallWildcardBeginA(cpArbiter *arb, cpSpace *space)
{
	cpCollisionHandler *handler = arb->handlerA;
	return handler->beginFunc(arb, space, handler->userData);
}

cpBool cpArbiterCallWildcardBeginB(cpArbiter *arb, cpSpace *space)
{
	cpCollisionHandler *handler = arb->handlerB;
	arb->swapped = !arb->swapped;
	cpBool retval = handler->beginFunc(arb, space, handler->userData);
	arb->swapped = !arb->swapped;
	return retval;
}

cpBool cpArbiterCallWildcardPreSolveA(cpArbiter *arb, cpSpace *space)
{
	cpCollisionHandler *handler = arb->handlerA;
	return handler->preSolveFunc(arb, space, handler->userData);
}

cpBool cpArbiterCallWildcardPreSolveB(cpArbiter *arb, cpSpace *space)
{
	cpCollisionHandler *handler = arb->handlerB;
	arb->swapped = !arb->swapped;
	cpBool retval = handler->preSolveFunc(arb, space, handler->userData);
	arb->swapped = !arb->swapped;
	return retval;
}

void cpArbiterCallWildcardPostSolveA(cpArbiter *arb, cpSpace *space)
{
	cpCollisionHandler *handler = arb->handlerA;
	handler->postSolveFunc(arb, space, handler->userData);
}

void cpArbiterCallWildcardPostSolveB(cpArbiter *arb, cpSpace *space)
{
	cpCollisionHandler *handler = arb->handlerB;
	arb->swapped = !arb->swapped;
	handler->postSolveFunc(arb, space, handler->userData);
	arb->swapped = !arb->swapped;
}

void cpArbiterCallWildcardSeparateA(cpArbiter *arb, cpSpace *space)
{
	cpCollisionHandler *handler = arb->handlerA;
	handler->separateFunc(arb, space, handler->userData);
}

void cpArbiterCallWildcardSeparateB(cpArbiter *arb, cpSpace *space)
{
	cpCollisionHandler *handler = arb->handlerB;
	arb->swapped = !arb->swapped;
	handler->separateFunc(arb, space, handler->userData);
	arb->swapped = !arb->swapped;
}

static cpBool default_begin_(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)data;
	cpBool retA = cpArbiterCallWildcardBeginA(arb, space);
	cpBool retB = cpArbiterCallWildcardBeginB(arb, space);
	return retA && retB;
}

static cpBool default_pre_solve_(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)data;
	cpBool retA = cpArbiterCallWildcardPreSolveA(arb, space);
	cpBool retB = cpArbiterCallWildcardPreSolveB(arb, space);
	return retA && retB;
}

static void default_post_solve_(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)data;
	cpArbiterCallWildcardPostSolveA(arb, space);
	cpArbiterCallWildcardPostSolveB(arb, space);
}

static void default_separate_(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)data;
	cpArbiterCallWildcardSeparateA(arb, space);
	cpArbiterCallWildcardSeparateB(arb, space);
}

static cpBool always_collide_(cpArbiter *arb, cpSpace *space, cpDataPointer data) { (void)arb; (void)space; (void)data; return cpTrue; }
static void do_nothing_(cpArbiter *arb, cpSpace *space, cpDataPointer data) { (void)arb; (void)space; (void)data; }

static cpCollisionHandler handler_default_ = {
	CP_WILDCARD_COLLISION_TYPE, CP_WILDCARD_COLLISION_TYPE,
	default_begin_, default_pre_solve_, default_post_solve_, default_separate_, NULL
};
static cpCollisionHandler handler_do_nothing_ = {
	CP_WILDCARD_COLLISION_TYPE, CP_WILDCARD_COLLISION_TYPE,
	always_collide_, always_collide_, do_nothing_, do_nothing_, NULL
};

/* cpSpaceLookupHandler (cpArbiter.c:348-354) */
static cpCollisionHandler *lookup_handler_(cpSpace *sp, cpCollisionType a, cpCollisionType b, cpCollisionHandler *def)
{
	for(int i = 0; i < sp->nhandlers; i++){
		cpCollisionHandler *h = sp->handlers[i];
		if((h->typeA == a && h->typeB == b) || (h->typeB == a && h->typeA == b)) return h;
	}
	return def;
}

static cpCollisionHandler *add_handler_(cpSpace *sp, const cpCollisionHandler *proto)
{
	sp->handlersOn = 1;
	sp->shapeDirty = 1;
	cpCollisionHandler *h = lookup_handler_(sp, proto->typeA, proto->typeB, NULL);
	if(h) return h;
	h = (cpCollisionHandler *)malloc(sizeof(cpCollisionHandler));
	memcpy(h, proto, sizeof(cpCollisionHandler));
	push_((void ***)&sp->handlers, &sp->nhandlers, &sp->caphandlers, h);
	return h;
}

static void use_wildcard_default_(cpSpace *sp)
{
	if(!sp->usesWildcards){
		sp->usesWildcards = 1;
		memcpy(&sp->defaultHandler, &handler_default_, sizeof(cpCollisionHandler));
	}
}

cpCollisionHandler *cpSpaceAddDefaultCollisionHandler(cpSpace *sp)
{
	use_wildcard_default_(sp);
	sp->handlersOn = 1;
	sp->defaultTouched = 1;
	sp->shapeDirty = 1;
	return &sp->defaultHandler;
}

cpCollisionHandler *cpSpaceAddCollisionHandler(cpSpace *sp, cpCollisionType a, cpCollisionType b)
{
	cpCollisionHandler proto = { a, b, default_begin_, default_pre_solve_, default_post_solve_, default_separate_, NULL };
	return add_handler_(sp, &proto);
}

cpCollisionHandler *cpSpaceAddWildcardHandler(cpSpace *sp, cpCollisionType type)
{
	use_wildcard_default_(sp);
	cpCollisionHandler proto = { type, CP_WILDCARD_COLLISION_TYPE, always_collide_, always_collide_, do_nothing_, do_nothing_, NULL };
	return add_handler_(sp, &proto);
}

/* cpArbiter.c:122-139, 174-238 */
cpBool cpArbiterIgnore(cpArbiter *arb) { arb->state = CPG_ARB_IGNORE; return cpFalse; }
void cpArbiterSetRestitution(cpArbiter *arb, cpFloat e) { arb->e = e; }
void cpArbiterSetFriction(cpArbiter *arb, cpFloat u) { arb->u = u; }
void cpArbiterSetSurfaceVelocity(cpArbiter *arb, cpVect vr) { arb->surface_vr = cpvmult(vr, arb->swapped ? -1.0 : 1.0); }
cpDataPointer cpArbiterGetUserData(const cpArbiter *arb) { return arb->data; }
void cpArbiterSetUserData(cpArbiter *arb, cpDataPointer data) { arb->data = data; }
cpBool cpArbiterIsRemoval(const cpArbiter *arb) { return arb->state == CPG_ARB_INVALIDATED; }

void cpArbiterSetContactPointSet(cpArbiter *arb, cpContactPointSet *set)
{
	int count = set->count;
	ASSERT_HARD(count == arb->count, "The number of contact points cannot be changed.");
	cpBool swapped = arb->swapped;
	arb->n = (swapped ? cpvneg(set->normal) : set->normal);
	for(int i = 0; i < count; i++){
		cpVect p1 = set->points[i].pointA, p2 = set->points[i].pointB;
		cpVect r1 = cpvsub(swapped ? p2 : p1, arb->body_a->p), r2 = cpvsub(swapped ? p1 : p2, arb->body_b->p);
		arb->c[i].r1x = r1.x; arb->c[i].r1y = r1.y;
		arb->c[i].r2x = r2.x; arb->c[i].r2y = r2.y;
	}
}

/* user data of the arbiters, by device key: an arbiter keeps its data
 * from update to update and a fresh one starts with none
 * (cpArbiter.c:343) */
static cpDataPointer *ud_slot_(cpSpace *sp, unsigned long long key, int insert)
{
	if(insert && 2*(sp->udUsed + 1) > sp->udCap){
		int oldCap = sp->udCap;
		unsigned long long *ok = sp->udKey;
		cpDataPointer *ov = sp->udVal;
		sp->udCap = oldCap ? 2*oldCap : 256;
		sp->udKey = (unsigned long long *)calloc((size_t)sp->udCap, sizeof(unsigned long long));
		sp->udVal = (cpDataPointer *)calloc((size_t)sp->udCap, sizeof(cpDataPointer));
		sp->udUsed = 0;
		for(int i = 0; i < oldCap; i++) if(ok[i]) *ud_slot_(sp, ok[i], 1) = ov[i];
		free(ok); free(ov);
	}
	if(sp->udCap == 0) return NULL;
	unsigned mask = (unsigned)sp->udCap - 1;
	unsigned h = (unsigned)((key*0x9e3779b97f4a7c15ull) >> 40) & mask;
	while(sp->udKey[h] && sp->udKey[h] != key) h = (h + 1) & mask;
	if(!sp->udKey[h]){
		if(!insert) return NULL;
		sp->udKey[h] = key;
		sp->udUsed++;
	}
	return &sp->udVal[h];
}

/* A device record as the callbacks' arbiter, with the handlers of its
 * types in update order (cpArbiter.c:399-410). */
/* fresh: the record is this step's update, where a new arbiter starts
 * without user data */
static void harb_fill_(cpSpace *sp, cpArbiter *arb, const cpgArb *g, int slot, int fresh)
{
	memset(arb, 0, sizeof(*arb));
	arb->a = sp->shapes[g->a]; arb->b = sp->shapes[g->b];
	arb->body_a = arb->a->body; arb->body_b = arb->b->body;
	arb->count = g->count; arb->state = g->state;
	arb->n = cpv(g->nx, g->ny); arb->surface_vr = cpv(g->svx, g->svy);
	arb->e = g->e; arb->u = g->u;
	arb->c[0] = g->c[0]; arb->c[1] = g->c[1];
	arb->key = garb_key_(g->a, g->b);
	arb->slot = slot;
	arb->listPos = -1;
	cpCollisionType typeA = arb->a->ctype, typeB = arb->b->ctype;
	cpCollisionHandler *defaultHandler = &sp->defaultHandler;
	cpCollisionHandler *handler = arb->handler = lookup_handler_(sp, typeA, typeB, defaultHandler);
	cpBool swapped = arb->swapped = (typeA != handler->typeA && handler->typeA != CP_WILDCARD_COLLISION_TYPE);
	arb->handlerA = arb->handlerB = &handler_do_nothing_;
	if(handler != defaultHandler || sp->usesWildcards){
		arb->handlerA = lookup_handler_(sp, (swapped ? typeB : typeA), CP_WILDCARD_COLLISION_TYPE, &handler_do_nothing_);
		arb->handlerB = lookup_handler_(sp, (swapped ? typeA : typeB), CP_WILDCARD_COLLISION_TYPE, &handler_do_nothing_);
	}
	if(fresh && (g->pad & CPG_ARB_FRESH)){
		cpDataPointer *ud = ud_slot_(sp, arb->key, 0);
		if(ud) *ud = NULL;
	} else {
		cpDataPointer *ud = ud_slot_(sp, arb->key, 0);
		arb->data = ud ? *ud : NULL;
	}
}

static void harb_keep_data_(cpSpace *sp, const cpArbiter *arb)
{
	cpDataPointer *ud = ud_slot_(sp, arb->key, arb->data != NULL);
	if(ud) *ud = arb->data;
}

static void harb_reserve_(cpSpace *sp, int n)
{
	if(n > sp->capharb){
		sp->capharb = n + n/2 + 16;
		sp->harb = (cpArbiter *)realloc(sp->harb, sizeof(cpArbiter)*(size_t)sp->capharb);
	}
}

static int bridge_buf_(DevSet *ds, int n)
{
	if(ds->bridgeCap >= n) return 1;
	if(ds->bridgeBuf) cudaFree(ds->bridgeBuf);
	ds->bridgeBuf = NULL; ds->bridgeCap = 0;
	if(!cuda_ok(cudaMalloc((void **)&ds->bridgeBuf, sizeof(int)*(size_t)n), "cudaMalloc handler buffers")) return 0;
	ds->bridgeCap = n;
	return 1;
}

/* Records by slot from the device. */
static cpgArb *gather_slots_(DevSet *ds, const int *hslots, int n)
{
	cpgArb *recs = HALLOC(cpgArb, n);
	if(n == 0) return recs;
	if(n > ds->gatherCap){
		if(ds->gather) cudaFree(ds->gather);
		ds->gatherCap = n + n/2 + 64;
		if(!cuda_ok(cudaMalloc((void **)&ds->gather, sizeof(cpgArb)*(size_t)ds->gatherCap), "gather")){ ds->gatherCap = 0; ds->gather = NULL; free(recs); return NULL; }
	}
	if(!bridge_buf_(ds, ds->d.arbCap + n + 1)){ free(recs); return NULL; }
	int *dslots = ds->bridgeBuf + ds->d.arbCap + 1;
	int ok = h2d(dslots, hslots, sizeof(int)*(size_t)n);
	ok &= cpg_launch_gather_slots(&ds->d, dslots, ds->gather, n, lib_stream()) == 0;
	ok &= d2h(recs, ds->gather, sizeof(cpgArb)*(size_t)n);
	ok &= cuda_ok(cudaStreamSynchronize(lib_stream()), "gather slots");
	if(!ok){ free(recs); return NULL; }
	return recs;
}

static void cpgarb_from_(cpgArb *g, const cpArbiter *arb)
{
	g->count = arb->count; g->state = arb->state;
	g->nx = arb->n.x; g->ny = arb->n.y;
	g->svx = arb->surface_vr.x; g->svy = arb->surface_vr.y;
	g->e = arb->e; g->u = arb->u;
	g->c[0] = arb->c[0]; g->c[1] = arb->c[1];
}

/* begin and pre-solve on the step's colliding arbiters of handled types,
 * in order (cpSpaceStep.c:259-286); the rule; the records and the list
 * back.  The list holds them among the arbiters the device kept by the
 * rule alone (their handlers do nothing). */
static int handlers_collide_(cpSpace *sp)
{
	DevSet *ds = sp->dev;
	const cpgWorld *W = &ds->hworld[sp->world];
	int n = 0;
	int *pairs = gather_pairs_(sp, &n);
	if(!pairs) return 0;
	int *slots = HALLOC(int, n);
	if(n > 0 && (!d2h(slots, ds->d.arbList + W->candOff, sizeof(int)*(size_t)n) ||
	             !cuda_ok(cudaStreamSynchronize(lib_stream()), "list slots"))){ free(pairs); free(slots); return 0; }
	/* the entries whose types have handlers */
	int *hidx = HALLOC(int, n), *hslots = HALLOC(int, n);
	int nh = 0;
	for(int i = 0; i < n; i++){
		cpShape *a = sp->shapes[pairs[2*i]], *b = sp->shapes[pairs[2*i + 1]];
		if(shape_needs_host_(sp, a) || shape_needs_host_(sp, b)){ hidx[nh] = i; hslots[nh] = slots[i]; nh++; }
	}
	cpgArb *recs = gather_slots_(ds, hslots, nh);
	if(!recs){ free(pairs); free(slots); free(hidx); free(hslots); return 0; }
	space_pull(sp);
	harb_reserve_(sp, nh);
	unsigned char *drop = HALLOC(unsigned char, n);
	sp->locked++;
	for(int k = 0; k < nh; k++){
		cpArbiter *arb = &sp->harb[k];
		harb_fill_(sp, arb, &recs[k], hslots[k], 1);
		cpCollisionHandler *handler = arb->handler;
		if(arb->state == CPG_ARB_FIRST && !handler->beginFunc(arb, sp, handler->userData)) cpArbiterIgnore(arb);
		cpShape *a = arb->a, *b = arb->b;
		if(!(arb->state != CPG_ARB_IGNORE && handler->preSolveFunc(arb, sp, handler->userData) && arb->state != CPG_ARB_IGNORE &&
		     !(a->sensor || b->sensor) && !(a->body->m == INF_ && b->body->m == INF_))){
			arb->count = 0;
			if(arb->state != CPG_ARB_IGNORE) arb->state = CPG_ARB_NORMAL;
			drop[hidx[k]] = 1;
		}
		harb_keep_data_(sp, arb);
		cpgarb_from_(&recs[k], arb);
	}
	/* the records back, then the list */
	unsigned long long *keep = HALLOC(unsigned long long, n);
	int nkeep = 0;
	for(int i = 0; i < n; i++) if(!drop[i]) keep[nkeep++] = garb_key_(pairs[2*i], pairs[2*i + 1]);
	int ok = 1;
	if(nh > 0){
		if(!bridge_buf_(ds, ds->d.arbCap + nh + 1)) ok = 0;
		else {
			int *dslots = ds->bridgeBuf + ds->d.arbCap + 1;
			ok &= h2d(dslots, hslots, sizeof(int)*(size_t)nh);
			ok &= h2d(ds->gather, recs, sizeof(cpgArb)*(size_t)nh);
			ok &= cpg_launch_put_arbs(&ds->d, dslots, ds->gather, nh, lib_stream()) == 0;
		}
	}
	if(ok){
		size_t lb = align256(sizeof(unsigned long long)*(size_t)(nkeep + 1));
		if(ds->qbytes < lb){
			if(ds->qbuf) cudaFree(ds->qbuf);
			ds->qbuf = NULL; ds->qbytes = 0;
			ok = cuda_ok(cudaMalloc(&ds->qbuf, lb), "cudaMalloc handler list");
			if(ok) ds->qbytes = lb;
		}
		if(ok){
			if(nkeep > 0) ok &= h2d(ds->qbuf, keep, sizeof(unsigned long long)*(size_t)nkeep);
			ok &= cpg_launch_sleep_edits(&ds->d, NULL, NULL, NULL, 0, (const unsigned long long *)ds->qbuf, nkeep, lib_stream()) == 0;
			ok &= cuda_ok(cudaStreamSynchronize(lib_stream()), "handler list");
		}
	}
	free(recs); free(pairs); free(slots); free(hidx); free(hslots); free(keep); free(drop);
	/* cpSpaceStep.c:373 */
	space_unlock_(sp);
	return ok;
}

/* separate on the arbiters the cache filter moved to the cached state
 * (cpSpaceStep.c:307-313), in slot order (the reference's is its hash
 * set's). */
static int cmp_int_(const void *x, const void *y) { int a = *(const int *)x, b = *(const int *)y; return (a > b) - (a < b); }

static int handlers_separate_(cpSpace *sp)
{
	DevSet *ds = sp->dev;
	int n = 0;
	if(!d2h(&n, ds->bridgeBuf + ds->d.arbCap, sizeof(int)) || !cuda_ok(cudaStreamSynchronize(lib_stream()), "separations")) return 0;
	if(n > ds->d.arbCap) n = ds->d.arbCap;
	if(n == 0) return 1;
	int *slots = HALLOC(int, n);
	if(!d2h(slots, ds->bridgeBuf, sizeof(int)*(size_t)n) || !cuda_ok(cudaStreamSynchronize(lib_stream()), "separations")){ free(slots); return 0; }
	qsort(slots, (size_t)n, sizeof(int), cmp_int_);
	cpgArb *recs = gather_slots_(ds, slots, n);
	if(!recs){ free(slots); return 0; }
	harb_reserve_(sp, n);
	sp->locked++;
	for(int i = 0; i < n; i++){
		if(recs[i].a < 0 || recs[i].a >= sp->nshapes || recs[i].b < 0 || recs[i].b >= sp->nshapes || !sp->shapes[recs[i].a] || !sp->shapes[recs[i].b]) continue;
		if(!shape_needs_host_(sp, sp->shapes[recs[i].a]) && !shape_needs_host_(sp, sp->shapes[recs[i].b])) continue;
		cpArbiter *arb = &sp->harb[i];
		harb_fill_(sp, arb, &recs[i], slots[i], 0);
		arb->handler->separateFunc(arb, sp, arb->handler->userData);
		harb_keep_data_(sp, arb);
	}
	space_unlock_(sp);
	free(recs); free(slots);
	return 1;
}

/* post-solve on the list with the solved impulses (cpSpaceStep.c:439-444) */
static int handlers_post_solve_(cpSpace *sp)
{
	DevSet *ds = sp->dev;
	const cpgWorld *W = &ds->hworld[sp->world];
	int n = 0;
	int *pairs = gather_pairs_(sp, &n);
	if(!pairs) return 0;
	int *slots = HALLOC(int, n);
	if(n > 0 && (!d2h(slots, ds->d.arbList + W->candOff, sizeof(int)*(size_t)n) ||
	             !cuda_ok(cudaStreamSynchronize(lib_stream()), "list slots"))){ free(pairs); free(slots); return 0; }
	int nh = 0;
	for(int i = 0; i < n; i++){
		cpShape *a = sp->shapes[pairs[2*i]], *b = sp->shapes[pairs[2*i + 1]];
		if(shape_needs_host_(sp, a) || shape_needs_host_(sp, b)) slots[nh++] = slots[i];
	}
	free(pairs);
	cpgArb *recs = gather_slots_(ds, slots, nh);
	if(!recs){ free(slots); return 0; }
	space_pull(sp);
	harb_reserve_(sp, nh);
	sp->locked++;
	for(int i = 0; i < nh; i++){
		cpArbiter *arb = &sp->harb[i];
		harb_fill_(sp, arb, &recs[i], -1, 0);
		arb->handler->postSolveFunc(arb, sp, arb->handler->userData);
		harb_keep_data_(sp, arb);
	}
	space_unlock_(sp);
	free(recs); free(slots);
	return 1;
}

/* cpSpace.c:490-503 on removal: the shape's cached arbiters, unless
 * already separated, are invalidated and separated. */
static void handlers_remove_shape_(cpSpace *sp, cpShape *s)
{
	if(!sp->handlersOn || !sp->dev || !sp->ownsDev) return;
	DevSet *ds = sp->dev;
	if(!bridge_buf_(ds, 2*(ds->d.arbCap + 1))) return;
	int *dslots = ds->bridgeBuf + ds->d.arbCap + 1, n = 0;
	if(cpg_launch_shape_arbs(&ds->d, (int)s->hashid, dslots, ds->bridgeBuf + ds->d.arbCap, ds->d.arbCap, lib_stream()) != 0) return;
	if(!d2h(&n, ds->bridgeBuf + ds->d.arbCap, sizeof(int)) || !cuda_ok(cudaStreamSynchronize(lib_stream()), "shape arbiters")) return;
	if(n > ds->d.arbCap) n = ds->d.arbCap;
	if(n == 0) return;
	int *slots = HALLOC(int, n);
	if(!d2h(slots, dslots, sizeof(int)*(size_t)n) || !cuda_ok(cudaStreamSynchronize(lib_stream()), "shape arbiters")){ free(slots); return; }
	qsort(slots, (size_t)n, sizeof(int), cmp_int_);
	cpgArb *recs = gather_slots_(ds, slots, n);
	if(!recs){ free(slots); return; }
	harb_reserve_(sp, n);
	sp->locked++;
	for(int i = 0; i < n; i++){
		if(recs[i].state == CPG_ARB_CACHED) continue;
		if(recs[i].a < 0 || recs[i].a >= sp->nshapes || recs[i].b < 0 || recs[i].b >= sp->nshapes || !sp->shapes[recs[i].a] || !sp->shapes[recs[i].b]) continue;
		cpArbiter *arb = &sp->harb[i];
		harb_fill_(sp, arb, &recs[i], slots[i], 0);
		arb->state = CPG_ARB_INVALIDATED;
		arb->handler->separateFunc(arb, sp, arb->handler->userData);
	}
	space_unlock_(sp);
	free(recs); free(slots);
}

/* cpSpace.c:662-678: the shape's cache brought to its body's transform,
 * then its leaf re-indexed (cpBBTreeReindexObject, replayed on the device
 * before the next step or query with the box and velocity of this call). */
void cpSpaceReindexShape(cpSpace *sp, cpShape *s)
{
	if(s->space != sp){
		/* not in this space: the reference finds no leaf and only caches */
		cpShapeCacheBB(s);
		return;
	}
	/* the whole state comes home first (space_detach): the new cache is
	 * what the rebuild uploads */
	if(!space_edit_ok(sp)) return;
	rd(s->body);
	shape_cache_(s, s->body->transform);
	/* a sleeping body's shapes are in the static index */
	record_op_(sp, CPG_OP_REINDEX, s, body_type_(s->body) == CP_BODY_TYPE_STATIC || cpBodyIsSleeping(s->body));
	sp->structDirty = 1;
	sp->editGen++;
}

void cpSpaceReindexShapesForBody(cpSpace *sp, cpBody *body)
{
	/* cpSpace.c:674-678, in the body's shape-list order */
	for(cpShape *s = body->shapeList; s; s = s->next) cpSpaceReindexShape(sp, s);
}

/* cpSpace.c:654-660: every static shape's cache updated, then the static
 * tree re-indexed as a whole (replayed on the device). */
void cpSpaceReindexStatic(cpSpace *sp)
{
	if(!space_edit_ok(sp)) return;
	for(int i = 0; i < sp->nshapes; i++){
		cpShape *s = sp->shapes[i];
		if(!s || body_type_(s->body) != CP_BODY_TYPE_STATIC) continue;
		shape_cache_(s, s->body->transform);
	}
	if(sp->nops == sp->capops){
		sp->capops = sp->capops ? 2*sp->capops : 256;
		sp->ops = (cpgOp *)realloc(sp->ops, sizeof(cpgOp)*(size_t)sp->capops);
	}
	cpgOp *op = &sp->ops[sp->nops++];
	memset(op, 0, sizeof(*op));
	op->kind = CPG_OP_REINDEX_STATIC;
	op->isStatic = 1;
	sp->structDirty = 1;
	sp->editGen++;
}

/* cpSpace.c:687-701: both indices become spatial hashes of cells of size
 * dim, next_prime(count) cells each, holding the same shapes (replayed on
 * the device as one edit, in call order with the others). */
void cpSpaceUseSpatialHash(cpSpace *sp, cpFloat dim, int count)
{
	if(!space_edit_ok(sp)) return;
	sp->useHash = 1;
	sp->hashDim = dim;
	sp->hashCells = (int)next_prime((unsigned)count);
	if(sp->nops == sp->capops){
		sp->capops = sp->capops ? 2*sp->capops : 256;
		sp->ops = (cpgOp *)realloc(sp->ops, sizeof(cpgOp)*(size_t)sp->capops);
	}
	cpgOp *op = &sp->ops[sp->nops++];
	memset(op, 0, sizeof(*op));
	op->kind = CPG_OP_USE_HASH;
	sp->structDirty = 1;
	sp->editGen++;
}

cpBody *cpSpaceAddBody(cpSpace *sp, cpBody *b)
{
	/* cpSpace.c:440-451 */
	ASSERT_HARD(b->space != sp, "You have already added this body to this space. You must not add it a second time.");
	ASSERT_HARD(!b->space, "You have already added this body to another space. You cannot add it to a second.");
	ASSERT_HARD(!sp->locked, "This operation cannot be done safely during a call to cpSpaceStep() or during a query. Put these calls into a post-step callback.");
	if(!space_edit_ok(sp)) return b;
	if(body_type_(b) == CP_BODY_TYPE_STATIC) push_((void ***)&sp->stat, &sp->nstat, &sp->capstat, b);
	else push_((void ***)&sp->dyn, &sp->ndyn, &sp->capdyn, b);
	b->space = sp;
	return b;
}

cpShape *cpSpaceAddShape(cpSpace *sp, cpShape *s)
{
	/* cpSpace.c:417-438 */
	ASSERT_HARD(s->space != sp, "You have already added this shape to this space. You must not add it a second time.");
	ASSERT_HARD(!s->space, "You have already added this shape to another space. You cannot add it to a second.");
	ASSERT_HARD(s->body, "The shape's body is not defined.");
	ASSERT_HARD(s->body->space == sp, "The shape's body must be added to the space before the shape.");
	ASSERT_HARD(!sp->locked, "This operation cannot be done safely during a call to cpSpaceStep() or during a query. Put these calls into a post-step callback.");
	if(!space_edit_ok(sp)) return s;
	cpBody *body = s->body;
	rd(body);
	int isStatic = (body_type_(body) == CP_BODY_TYPE_STATIC);
	if(!isStatic) cpBodyActivate(body);
	cpShape *next = body->shapeList;
	if(next) next->prev = s;
	s->next = next;
	body->shapeList = s;
	if(s->mass_m > 0.0) accumulate_mass_(body);
	/* the hash id is the shape's slot: ids are never reused */
	s->hashid = sp->shapeIDCounter++;
	shape_cache_(s, body->transform);
	record_op_(sp, CPG_OP_INSERT, s, isStatic);
	push_((void ***)&sp->shapes, &sp->nshapes, &sp->capshapes, s);
	sp->nlive++;
	s->space = sp;
	return s;
}

cpConstraint *cpSpaceAddConstraint(cpSpace *sp, cpConstraint *c)
{
	/* cpSpace.c:453-474 */
	ASSERT_HARD(c->space != sp, "You have already added this constraint to this space. You must not add it a second time.");
	ASSERT_HARD(!c->space, "You have already added this constraint to another space. You cannot add it to a second.");
	ASSERT_HARD(c->a != NULL && c->b != NULL, "Constraint is attached to a NULL body.");
	ASSERT_HARD(!sp->locked, "This operation cannot be done safely during a call to cpSpaceStep() or during a query. Put these calls into a post-step callback.");
	if(!space_edit_ok(sp)) return c;
	cpBody *a = c->a, *b = c->b;
	cpBodyActivate(a);
	cpBodyActivate(b);
	c->index = sp->ncons;
	push_((void ***)&sp->cons, &sp->ncons, &sp->capcons, c);
	c->next_a = a->constraintList; a->constraintList = c;
	c->next_b = b->constraintList; b->constraintList = c;
	c->space = sp;
	return c;
}

void cpSpaceRemoveShape(cpSpace *sp, cpShape *s)
{
	/* cpSpace.c:523-545 */
	ASSERT_HARD(cpSpaceContainsShape(sp, s), "Cannot remove a shape that was not added to the space. (Removed twice maybe?)");
	ASSERT_HARD(!sp->locked, "This operation cannot be done safely during a call to cpSpaceStep() or during a query. Put these calls into a post-step callback.");
	if(!space_edit_ok(sp)) return;
	cpBody *body = s->body;
	int isStatic = (body_type_(body) == CP_BODY_TYPE_STATIC);
	if(isStatic) cpBodyActivateStatic(body, s);
	else cpBodyActivate(body);
	handlers_remove_shape_(sp, s);
	/* the shape's arbiters leave the contact graph and the list
	 * (cachedArbitersFilter, cpSpace.c:481-512) */
	if(sp->graphOn){
		for(int g = 0; g < sp->ngarb; g++){
			cpArbiter *arb = &sp->garb[g];
			if(!arb->a || (arb->a != s && arb->b != s)) continue;
			/* its pending cache edits go with it */
			int k = 0;
			for(int i = 0; i < sp->nsed; i++){
				if(sp->sedKey[i] == arb->key) continue;
				sp->sedKey[k] = sp->sedKey[i]; sp->sedOp[k] = sp->sedOp[i]; sp->sedStamp[k] = sp->sedStamp[i]; k++;
			}
			sp->nsed = k;
			gunthread_(sp, g);
			glist_delete_(sp, g);
			garb_release_(sp, g);
		}
	}
	/* cpBodyRemoveShape, cpBody.c:306-327 */
	if(s->prev) s->prev->next = s->next; else body->shapeList = s->next;
	if(s->next) s->next->prev = s->prev;
	s->prev = s->next = NULL;
	if(body_type_(body) == CP_BODY_TYPE_DYNAMIC && s->mass_m > 0.0) accumulate_mass_(body);
	/* its arbiters go when the set is rebuilt (cpSpaceFilterArbiters), its
	 * leaf when the edit replays (cpSpatialIndexRemove) */
	record_op_(sp, CPG_OP_REMOVE, s, isStatic);
	sp->shapes[s->hashid] = NULL;
	sp->nlive--;
	s->space = NULL;
	s->hashid = 0;
}

void cpSpaceRemoveBody(cpSpace *sp, cpBody *b)
{
	/* cpSpace.c:547-562 */
	ASSERT_HARD(b != cpSpaceGetStaticBody(sp), "Cannot remove the designated static body for the space.");
	ASSERT_HARD(cpSpaceContainsBody(sp, b), "Cannot remove a body that was not added to the space. (Removed twice maybe?)");
	ASSERT_HARD(!sp->locked, "This operation cannot be done safely during a call to cpSpaceStep() or during a query. Put these calls into a post-step callback.");
	if(!space_edit_ok(sp)) return;
	cpBodyActivate(b);
	if(body_type_(b) == CP_BODY_TYPE_STATIC) array_delete_((void **)sp->stat, &sp->nstat, b);
	else array_delete_((void **)sp->dyn, &sp->ndyn, b);
	b->space = NULL;
}

/* cpBody.c:272-287 (filterConstraints), iteratively */
static void body_remove_constraint_(cpBody *body, cpConstraint *c)
{
	cpConstraint **link = &body->constraintList;
	int guard = 0;
	while(*link && guard++ < (1 << 30)){
		cpConstraint *node = *link;
		if(node == c){ *link = cons_next_(node, body); return; }
		link = (node->a == body) ? &node->next_a : &node->next_b;
	}
}

void cpSpaceRemoveConstraint(cpSpace *sp, cpConstraint *c)
{
	/* cpSpace.c:564-577: the constraint array loses it like
	 * cpArrayDeleteObj, so the last constraint takes its place in the
	 * solve order */
	ASSERT_HARD(cpSpaceContainsConstraint(sp, c), "Cannot remove a constraint that was not added to the space. (Removed twice maybe?)");
	ASSERT_HARD(!sp->locked, "This operation cannot be done safely during a call to cpSpaceStep() or during a query. Put these calls into a post-step callback.");
	if(!space_edit_ok(sp)) return;
	cpBodyActivate(c->a);
	cpBodyActivate(c->b);
	int i = array_delete_((void **)sp->cons, &sp->ncons, c);
	if(i >= 0 && i < sp->ncons) sp->cons[i]->index = i;
	body_remove_constraint_(c->a, c);
	body_remove_constraint_(c->b, c);
	c->space = NULL;
	c->index = -1;
}

/* cpSpace.c:589-617: the dynamic array, the static array, then each
 * sleeping component from its root */
void cpSpaceEachBody(cpSpace *sp, cpSpaceBodyIteratorFunc func, void *data)
{
	sp->locked++;
	for(int i = 0; i < sp->ndyn; i++) func(sp->dyn[i], data);
	for(int i = 0; i < sp->nstat; i++) func(sp->stat[i], data);
	for(int i = 0; i < sp->nsleeping; i++){
		cpBody *b = sp->sleeping[i];
		while(b){
			cpBody *next = b->sleepNext;
			func(b, data);
			b = next;
		}
	}
	space_unlock_(sp);
	run_post_step_(sp);
}

/* cpSpace.c:621-629: the dynamic then the static index's leaves, each in
 * its leaf hash set's order (bins, then each bin's chain: cpHashSet.c),
 * which the device sets keep as the reference's do. */
void cpSpaceEachShape(cpSpace *sp, cpSpaceShapeIteratorFunc func, void *data)
{
	if(!sp) return;
	if(sp->nshapes > 0 && !(sp->dev && !sp->ownsDev && (sp->structDirty || space_structure_changed(sp))) &&
	   (sp->dev && !sp->ownsDev ? 1 : space_device_ready_(sp))){
		DevSet *ds = sp->dev;
		const cpgWorld *W = &ds->hworld[sp->world];
		cpgTree T;
		int nn = W->nodeCap;
		int *bins = HALLOC(int, (size_t)W->dbinCap + (size_t)W->sbinCap);
		cpgNode *nodes = HALLOC(cpgNode, nn);
		int ok = d2h(&T, ds->d.tree + sp->world, sizeof(cpgTree));
		ok &= d2h(bins, ds->d.dbins + W->dbinOff, sizeof(int)*(size_t)W->dbinCap);
		ok &= d2h(bins + W->dbinCap, ds->d.sbins + W->sbinOff, sizeof(int)*(size_t)W->sbinCap);
		ok &= d2h(nodes, ds->d.nodes + W->nodeOff, sizeof(cpgNode)*(size_t)nn);
		ok &= cuda_ok(cudaStreamSynchronize(lib_stream()), "shape iteration");
		if(ok){
			int nshapes = sp->nshapes;
			cpShape **order = HALLOC(cpShape *, nshapes);
			int n = 0;
			for(int set = 0; set < 2; set++){
				const int *b = set ? bins + W->dbinCap : bins;
				unsigned size = set ? T.statSize : T.dynSize;
				int cap = set ? W->sbinCap : W->dbinCap;
				for(unsigned i = 0; i < size && (int)i < cap; i++){
					int guard = 0;
					for(int k = b[i]; k >= 0 && k < nn && guard <= nn; k = nodes[k].binNext, guard++){
						cpShape *shape = slot_shape_(sp, nodes[k].obj);
						if(shape && n < nshapes) order[n++] = shape;
					}
				}
			}
			/* iterate a copy taken before the first callback */
			sp->locked++;
			for(int i = 0; i < n; i++) func(order[i], data);
			space_unlock_(sp);
			free(order);
			free(bins); free(nodes);
			run_post_step_(sp);
			return;
		}
		free(bins); free(nodes);
	}
	sp->locked++;
	for(int i = 0; i < sp->nshapes; i++) if(sp->shapes[i]) func(sp->shapes[i], data);
	space_unlock_(sp);
	run_post_step_(sp);
}

void cpSpaceEachConstraint(cpSpace *sp, cpSpaceConstraintIteratorFunc func, void *data)
{
	sp->locked++;
	for(int i = 0; i < sp->ncons; i++) func(sp->cons[i], data);
	space_unlock_(sp);
	run_post_step_(sp);
}

/* cpSpaceStep.c:26-58, 84-103: post-step callbacks, one per key, run in
 * the order added when the step (or an iteration or query) ends; a
 * callback added by one of them runs in the same round. */
typedef struct PostStep { cpPostStepFunc func; void *key, *data; } PostStep;

cpBool cpSpaceAddPostStepCallback(cpSpace *sp, cpPostStepFunc func, void *key, void *data)
{
	for(int i = 0; i < sp->npost; i++) if(sp->post[i].key == key) return cpFalse;
	if(sp->npost == sp->cappost){
		sp->cappost = sp->cappost ? 2*sp->cappost : 8;
		sp->post = (PostStep *)realloc(sp->post, sizeof(PostStep)*(size_t)sp->cappost);
	}
	PostStep *cb = &sp->post[sp->npost++];
	cb->func = func; cb->key = key; cb->data = data;
	return cpTrue;
}

static void run_post_step_(cpSpace *sp)
{
	if(!sp || sp->postRunning || sp->npost == 0) return;
	sp->postRunning = 1;
	for(int i = 0; i < sp->npost; i++){
		PostStep cb = sp->post[i];
		sp->post[i].func = NULL;
		if(cb.func) cb.func(sp, cb.key, cb.data);
	}
	sp->npost = 0;
	sp->postRunning = 0;
}

/* ====================================================================
 * Arbiters: snapshot of the solve list (cpArbiter.c:54-155)
 * ==================================================================== */
static int space_snapshot(cpSpace *sp)
{
	if(sp->snapValid) return 1;
	sp->nsnap = 0;
	if(!sp->dev){ sp->snapValid = 1; return 1; }
	space_pull(sp);
	DevSet *ds = sp->dev;
	cpgTree T;
	d2h(&T, ds->d.tree + sp->world, sizeof(cpgTree));
	cudaStreamSynchronize(lib_stream());
	int n = T.narb;
	if(n > ds->gatherCap){
		if(ds->gather) cudaFree(ds->gather);
		ds->gatherCap = n + n/2 + 64;
		if(!cuda_ok(cudaMalloc((void **)&ds->gather, sizeof(cpgArb)*(size_t)ds->gatherCap), "gather")) { ds->gatherCap = 0; ds->gather = NULL; return 0; }
	}
	cpgArb *host = HALLOC(cpgArb, n);
	if(n > 0){
		cpg_launch_gather_arbs(&ds->d, sp->world, ds->gather, n, lib_stream());
		d2h(host, ds->gather, sizeof(cpgArb)*(size_t)n);
		cudaStreamSynchronize(lib_stream());
	}
	if(n > sp->capsnap){
		sp->capsnap = n + 64;
		sp->snap = (cpArbiter *)realloc(sp->snap, sizeof(cpArbiter)*(size_t)sp->capsnap);
	}
	int kept = 0;
	for(int i = 0; i < n; i++){
		cpgArb *g = &host[i];
		/* a shape removed since the step: its arbiters are gone too
		 * (cpSpaceFilterArbiters) */
		if(g->a < 0 || g->a >= sp->nshapes || g->b < 0 || g->b >= sp->nshapes || !sp->shapes[g->a] || !sp->shapes[g->b]) continue;
		cpArbiter *arb = &sp->snap[kept++];
		arb->a = sp->shapes[g->a]; arb->b = sp->shapes[g->b];
		arb->body_a = arb->a->body; arb->body_b = arb->b->body;
		arb->count = g->count; arb->state = g->state;
		arb->n = cpv(g->nx, g->ny); arb->surface_vr = cpv(g->svx, g->svy);
		arb->e = g->e; arb->u = g->u; arb->swapped = cpFalse;
		arb->c[0] = g->c[0]; arb->c[1] = g->c[1];
	}
	sp->nsnap = kept;
	sp->snapValid = 1;
	free(host);
	return 1;
}

int cpArbiterGetCount(const cpArbiter *arb) { return (arb->state < CPG_ARB_CACHED ? arb->count : 0); }
cpFloat cpArbiterGetRestitution(const cpArbiter *arb) { return arb->e; }
cpFloat cpArbiterGetFriction(const cpArbiter *arb) { return arb->u; }
cpVect cpArbiterGetSurfaceVelocity(cpArbiter *arb) { return cpvmult(arb->surface_vr, arb->swapped ? -1.0 : 1.0); }
cpBool cpArbiterIsFirstContact(const cpArbiter *arb) { return arb->state == CPG_ARB_FIRST; }
cpVect cpArbiterGetNormal(const cpArbiter *arb) { return cpvmult(arb->n, arb->swapped ? -1.0 : 1.0); }

cpVect cpArbiterGetPointA(const cpArbiter *arb, int i)
{
	ASSERT_HARD(0 <= i && i < cpArbiterGetCount(arb), "Index error: The specified contact index is invalid for this arbiter");
	return cpvadd(arb->body_a->p, cpv(arb->c[i].r1x, arb->c[i].r1y));
}

cpVect cpArbiterGetPointB(const cpArbiter *arb, int i)
{
	ASSERT_HARD(0 <= i && i < cpArbiterGetCount(arb), "Index error: The specified contact index is invalid for this arbiter");
	return cpvadd(arb->body_b->p, cpv(arb->c[i].r2x, arb->c[i].r2y));
}

cpFloat cpArbiterGetDepth(const cpArbiter *arb, int i)
{
	ASSERT_HARD(0 <= i && i < cpArbiterGetCount(arb), "Index error: The specified contact index is invalid for this arbiter");
	const cpgContact *con = &arb->c[i];
	return cpvdot(cpvadd(cpvsub(cpv(con->r2x, con->r2y), cpv(con->r1x, con->r1y)), cpvsub(arb->body_b->p, arb->body_a->p)), arb->n);
}

cpVect cpArbiterTotalImpulse(const cpArbiter *arb)
{
	cpVect n = arb->n, sum = cpvzero;
	for(int i = 0, count = cpArbiterGetCount(arb); i < count; i++){
		sum = cpvadd(sum, cpvrotate(n, cpv(arb->c[i].jnAcc, arb->c[i].jtAcc)));
	}
	return (arb->swapped ? sum : cpvneg(sum));
}

cpFloat cpArbiterTotalKE(const cpArbiter *arb)
{
	cpFloat eCoef = (1 - arb->e)/(1 + arb->e);
	cpFloat sum = 0.0;
	for(int i = 0, count = cpArbiterGetCount(arb); i < count; i++){
		const cpgContact *con = &arb->c[i];
		sum += eCoef*con->jnAcc*con->jnAcc/con->nMass + con->jtAcc*con->jtAcc/con->tMass;
	}
	return sum;
}

void cpArbiterGetShapes(const cpArbiter *arb, cpShape **a, cpShape **b)
{
	if(arb->swapped){ *a = arb->b; *b = arb->a; } else { *a = arb->a; *b = arb->b; }
}

void cpArbiterGetBodies(const cpArbiter *arb, cpBody **a, cpBody **b)
{
	cpShape *sa, *sb;
	cpArbiterGetShapes(arb, &sa, &sb);
	*a = sa->body; *b = sb->body;
}

cpContactPointSet cpArbiterGetContactPointSet(const cpArbiter *arb)
{
	cpContactPointSet set;
	memset(&set, 0, sizeof(set));
	set.count = cpArbiterGetCount(arb);
	cpBool swapped = arb->swapped;
	cpVect n = arb->n;
	set.normal = (swapped ? cpvneg(n) : n);
	for(int i = 0; i < set.count; i++){
		cpVect p1 = cpvadd(arb->body_a->p, cpv(arb->c[i].r1x, arb->c[i].r1y));
		cpVect p2 = cpvadd(arb->body_b->p, cpv(arb->c[i].r2x, arb->c[i].r2y));
		set.points[i].pointA = (swapped ? p2 : p1);
		set.points[i].pointB = (swapped ? p1 : p2);
		set.points[i].distance = cpvdot(cpvsub(p2, p1), n);
	}
	return set;
}

/* The contact graph threads each solved arbiter onto the head of both
 * bodies' lists (cpSpaceComponent.c:170-181), so a body sees its arbiters
 * in reverse solve order, with `swapped` relative to it (cpBody.c:612-626). */
void cpBodyEachArbiter(cpBody *body, cpBodyArbiterIteratorFunc func, void *data)
{
	cpSpace *sp = body->space;
	if(sp && sp->graphOn){
		/* cpBody.c:612-626 over the contact graph */
		graph_refresh_(sp);
		for(int k = body->arbList; k;){
			cpArbiter *arb = GARB_AT_(sp, k);
			int next = garb_next_(sp, k, body);
			cpBool swapped = arb->swapped;
			arb->swapped = (body == arb->body_b);
			func(body, arb, data);
			arb->swapped = swapped;
			k = next;
		}
		return;
	}
	if(!sp || !space_snapshot(sp)) return;
	for(int i = sp->nsnap - 1; i >= 0; i--){
		cpArbiter *arb = &sp->snap[i];
		if(arb->body_a != body && arb->body_b != body) continue;
		cpBool swapped = arb->swapped;
		arb->swapped = (body == arb->body_b);
		func(body, arb, data);
		arb->swapped = swapped;
	}
}

/* ====================================================================
 * Debug export (shared record layouts) and per-phase timing
 * ==================================================================== */
int cpGpuDebugBodies(cpSpace *sp, double *out, int max)
{
	space_pull(sp);
	for(int i = 0; i < sp->ndyn && i < max; i++){
		cpBody *b = sp->dyn[i];
		double *o = out + 18*i;
		o[0] = b->p.x; o[1] = b->p.y; o[2] = b->v.x; o[3] = b->v.y; o[4] = b->a; o[5] = b->w;
		o[6] = b->f.x; o[7] = b->f.y; o[8] = b->t; o[9] = b->v_bias.x; o[10] = b->v_bias.y; o[11] = b->w_bias;
		o[12] = b->transform.a; o[13] = b->transform.b; o[14] = b->transform.c; o[15] = b->transform.d;
		o[16] = b->transform.tx; o[17] = b->transform.ty;
	}
	return sp->ndyn;
}

int cpGpuDebugSetBodies(cpSpace *sp, const double *in, int count)
{
	space_pull(sp);
	for(int i = 0; i < sp->ndyn && i < count; i++){
		cpBody *b = sp->dyn[i];
		const double *o = in + 18*i;
		b->p = cpv(o[0], o[1]); b->v = cpv(o[2], o[3]); b->a = o[4]; b->w = o[5];
		b->f = cpv(o[6], o[7]); b->t = o[8]; b->v_bias = cpv(o[9], o[10]); b->w_bias = o[11];
		b->transform = cpTransformNew(o[12], o[13], o[14], o[15], o[16], o[17]);
	}
	sp->bodyDirty = 1;
	return sp->ndyn;
}

int cpGpuDebugSetImpulses(cpSpace *sp, const double *arbs, int narb, const double *cons, int ncons)
{
	int bad = 0;
	if(sp->dev && narb > 0){
		DevSet *ds = sp->dev;
		space_pull(sp);
		double *himp = HALLOC(double, 4*narb);
		int *hpair = HALLOC(int, 2*narb);
		for(int i = 0; i < narb; i++){
			const double *o = arbs + 34*i;
			hpair[2*i] = (int)o[0]; hpair[2*i + 1] = (int)o[1];
			himp[4*i] = o[17]; himp[4*i + 1] = o[18]; himp[4*i + 2] = o[29]; himp[4*i + 3] = o[30];
		}
		char *buf = NULL;
		size_t bi = sizeof(double)*4*(size_t)narb, bp = sizeof(int)*2*(size_t)narb;
		if(cuda_ok(cudaMalloc((void **)&buf, bi + bp + 16), "debug impulses")){
			cudaStream_t st = lib_stream();
			int *mis = (int *)(buf + bi + bp);
			int ok = h2d(buf, himp, bi) && h2d(buf + bi, hpair, bp) &&
				cuda_ok(cudaMemsetAsync(mis, 0, sizeof(int), st), "memset");
			if(ok && cpg_launch_set_arb_impulses(&ds->d, sp->world, (const double *)buf, (const int *)(buf + bi), narb, mis, st) == 0)
				d2h(&bad, mis, sizeof(int));
			cudaStreamSynchronize(st);
			cudaFree(buf);
		}
		free(himp); free(hpair);
		sp->snapValid = 0;
	}
	for(int i = 0; i < sp->ncons && i < ncons; i++){
		cpConstraint *c = sp->cons[i];
		const double *o = cons + 8*i;
		cons_pull_(c);
		if(c->kind == CPG_PIVOT || c->kind == CPG_GROOVE){ c->rec.jx = o[1]; c->rec.jy = o[2]; }
		else c->rec.jnAcc = o[1];
		if(c->kind == CPG_RATCHET) c->rec.angle = o[3];
		sp->consDirty = 1;
	}
	return bad;
}

/* Solver quality from the space's current state: the next step is run
 * from a saved copy of the device state once per iteration count k = 1 ..
 * maxIters (the first k iterations of a sweep do not depend on how many
 * follow), with solver mode `mode`; after each run the contacts' RMS normal
 * and friction residuals and the largest penetration are measured
 * (k_contact_quality), and the state is put back, so the space is left as
 * it was. */
int cpGpuSolverQuality(cpSpace *sp, int mode, cpFloat dt, int maxIters, double *out)
{
	if(!sp || !sp->dev || !sp->ownsDev || sp->structDirty || maxIters < 1 || !out || !(dt > 0.0) ||
	   mode < CP_GPU_SOLVER_ORDERED || mode > CP_GPU_SOLVER_COLORED){
		set_error(CP_GPU_ERR_ARGUMENT, "solver quality: a stepped standalone space, iterations >= 1 and dt > 0 are needed");
		return -1;
	}
	DevSet *ds = sp->dev;
	cudaStream_t st = lib_stream();
	devset_flush_space(ds, 0);
	char *saved = NULL;
	double *acc = NULL;
	if(!cuda_ok(cudaMalloc((void **)&saved, ds->slabBytes), "cudaMalloc quality state")) return -1;
	if(!cuda_ok(cudaMalloc((void **)&acc, 4*sizeof(double)), "cudaMalloc quality")){ cudaFree(saved); return -1; }
	cuda_ok(cudaMemcpyAsync(saved, ds->slab, ds->slabBytes, cudaMemcpyDeviceToDevice, st), "save state");
	unsigned stamp = sp->stamp;
	double currDt = sp->curr_dt, jointDt = sp->jointDt;
	int iters = sp->iterations, oldMode = sp->mode, rc = 0;
	for(int k = 1; k <= maxIters && rc == 0; k++){
		if(k > 1) rollout_restore_from(ds, saved, &stamp, &currDt);
		sp->jointDt = jointDt;
		sp->iterations = k;
		sp->mode = mode;
		double dts[1] = { dt };
		double h[4] = { 0.0, 0.0, 0.0, 0.0 };
		rc = devset_step(ds, dts, NULL);
		if(rc == 0 && cpg_launch_contact_quality(&ds->d, 0, dt, acc, st) != 0) rc = -1;
		if(rc == 0 && !d2h(h, acc, sizeof(h))) rc = -1;
		if(rc == 0 && !cuda_ok(cudaStreamSynchronize(st), "quality")) rc = -1;
		double n = h[2] > 0.0 ? h[2] : 1.0, pen;
		memcpy(&pen, &h[3], sizeof(pen));
		out[3*(k - 1)] = sqrt(h[0]/n);
		out[3*(k - 1) + 1] = sqrt(h[1]/n);
		out[3*(k - 1) + 2] = pen;
	}
	rollout_restore_from(ds, saved, &stamp, &currDt);
	sp->jointDt = jointDt;
	sp->iterations = iters;
	sp->mode = oldMode;
	cudaStreamSynchronize(st);
	check_stats(ds);
	cudaFree(saved);
	cudaFree(acc);
	return rc;
}

int cpGpuDebugNarrowIds(cpSpace *sp, int *out, int max)
{
	if(!sp || !sp->dev) return 0;
	DevSet *ds = sp->dev;
	space_pull(sp);
	cpgTree T;
	d2h(&T, ds->d.tree + sp->world, sizeof(cpgTree));
	cudaStreamSynchronize(lib_stream());
	int n = T.ncand;
	cpgCand *c = HALLOC(cpgCand, n);
	cpgNarrow *r = HALLOC(cpgNarrow, n);
	int off = ds->hworld[sp->world].candOff;
	d2h(c, ds->d.cands + off, sizeof(cpgCand)*(size_t)n);
	d2h(r, ds->d.narrow + off, sizeof(cpgNarrow)*(size_t)n);
	cudaStreamSynchronize(lib_stream());
	for(int i = 0; i < n && i < max; i++){
		out[4*i] = c[i].a; out[4*i + 1] = c[i].b; out[4*i + 2] = (int)c[i].idIn; out[4*i + 3] = (int)r[i].idOut;
	}
	free(c); free(r);
	return n;
}

int cpGpuDebugArbiters(cpSpace *sp, double *out, int max)
{
	if(!space_snapshot(sp)) return 0;
	for(int i = 0; i < sp->nsnap && i < max; i++){
		cpArbiter *arb = &sp->snap[i];
		double *o = out + 34*i;
		memset(o, 0, 34*sizeof(double));
		o[0] = (double)arb->a->hashid; o[1] = (double)arb->b->hashid; o[2] = arb->count; o[3] = arb->state;
		o[4] = arb->n.x; o[5] = arb->n.y; o[6] = arb->e; o[7] = arb->u; o[8] = arb->surface_vr.x; o[9] = arb->surface_vr.y;
		for(int c = 0; c < arb->count; c++){
			const cpgContact *con = &arb->c[c];
			double *q = o + 10 + 12*c;
			q[0] = con->r1x; q[1] = con->r1y; q[2] = con->r2x; q[3] = con->r2y;
			q[4] = con->nMass; q[5] = con->tMass; q[6] = con->bounce; q[7] = con->jnAcc; q[8] = con->jtAcc;
			q[9] = con->jBias; q[10] = con->bias; q[11] = (double)(con->hash & 0xffffffffffffULL);
		}
	}
	return sp->nsnap;
}

int cpGpuDebugConstraints(cpSpace *sp, double *out, int max)
{
	for(int i = 0; i < sp->ncons && i < max; i++){
		cpConstraint *c = sp->cons[i];
		cons_pull_(c);
		const cpgJoint *j = &c->rec;
		double *o = out + 8*i;
		memset(o, 0, 8*sizeof(double));
		o[0] = (double)c->kind;
		switch(c->kind){
		case CPG_PIVOT: case CPG_GROOVE: o[1] = j->jx; o[2] = j->jy; o[7] = j->biasx; break;
		case CPG_PIN: case CPG_SLIDE: o[1] = j->jnAcc; o[2] = j->nMass; o[7] = j->bias; break;
		case CPG_DSPRING: o[1] = j->jnAcc; o[2] = j->nMass; o[7] = j->coef; break;
		case CPG_DRSPRING: o[1] = j->jnAcc; o[2] = j->nMass; o[3] = j->coef; o[7] = j->bias; break;
		case CPG_RATCHET: o[1] = j->jnAcc; o[2] = j->nMass; o[3] = j->angle; o[7] = j->bias; break;
		case CPG_ROTLIMIT: case CPG_GEAR: o[1] = j->jnAcc; o[2] = j->nMass; o[7] = j->bias; break;
		default: o[1] = j->jnAcc; o[2] = j->nMass; break;
		}
		if(c->kind <= CPG_DSPRING){ o[3] = j->r1x; o[4] = j->r1y; o[5] = j->r2x; o[6] = j->r2y; }
	}
	return sp->ncons;
}

int cpGpuGetStepStats(cpSpace *sp, int *out, int max)
{
	if(!sp || !sp->dev || max < 1) return 0;
	DevSet *ds = sp->dev;
	/* the stats block of the last step: error flags, pair/node use (per
	 * mille of capacity), live arbiters, candidates, solved arbiters,
	 * sweep levels or colours, candidate use (per mille), leaves
	 * reinserted in the exact-order tree; the step's own asynchronous
	 * read-back may be older */
	check_stats(ds);
	if(!d2h(ds->hstats, ds->d.stats, sizeof(int)*16)) return 0;
	cudaStreamSynchronize(lib_stream());
	int n = max < 9 ? max : 9;
	for(int i = 0; i < n; i++) out[i] = ds->hstats[i];
	return n;
}

int cpGpuGetPhaseTimes(cpSpace *sp, double *ms, int max)
{
	for(int i = 0; i < 7 && i < max; i++) ms[i] = sp->phaseMs[i];
	return 7;
}

/* Shape-id pairs (min, max) of the last step's candidates whose boxes
 * intersect (the pair set the broadphase handed to the narrow phase). */
int cpGpuDebugCandidates(cpSpace *sp, int *out, int max)
{
	if(!sp->dev) return 0;
	DevSet *ds = sp->dev;
	cpgTree T;
	d2h(&T, ds->d.tree + sp->world, sizeof(cpgTree));
	cudaStreamSynchronize(lib_stream());
	int n = T.ncand;
	cpgCand *c = HALLOC(cpgCand, n);
	d2h(c, ds->d.cands + ds->hworld[sp->world].candOff, sizeof(cpgCand)*(size_t)n);
	cudaStreamSynchronize(lib_stream());
	space_pull(sp);
	int k = 0;
	for(int i = 0; i < n; i++){
		cpShape *a = sp->shapes[c[i].a], *b = sp->shapes[c[i].b];
		if(!a || !b) continue;
		cpBB ba = shape_bb_now_(a), bb = shape_bb_now_(b);
		if(!cpBBIntersects(ba, bb)) continue;
		if(k < max){
			int x = (int)a->hashid, y = (int)b->hashid;
			out[2*k] = x < y ? x : y; out[2*k + 1] = x < y ? y : x;
		}
		k++;
	}
	free(c);
	return k;
}


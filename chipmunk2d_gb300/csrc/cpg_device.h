/*
 * cpg_device.h -- device data layout shared by the C host code and the
 * CUDA kernels of libchipmunk_gb300.
 *
 * A "set" holds W independent worlds (a single cpSpace is a set of one;
 * cpGpuBatch packs thousands).  Every per-object array is the
 * concatenation of the worlds' ranges; cpgWorld gives each world's base
 * offsets and capacities.  All cross-references stored in device memory
 * (body of a shape, tree node links, pair links, arbiter shapes) are
 * world-local indices, so a world can be moved to a new base without
 * rewriting its contents.
 *
 * Plain C structs only: both gcc and nvcc compile this header and must
 * agree on every layout (all members are 4- or 8-byte scalars).
 */
#ifndef CPG_DEVICE_H
#define CPG_DEVICE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* shape kinds, in the collision-dispatch order of cpCollision.c:688-699 */
enum { CPG_CIRCLE = 0, CPG_SEGMENT = 1, CPG_POLY = 2 };
/* body types as cpBodyType */
enum { CPG_DYNAMIC = 0, CPG_KINEMATIC = 1, CPG_STATIC = 2 };
/* joint kinds */
enum { CPG_PIVOT = 1, CPG_PIN = 2, CPG_SLIDE = 3, CPG_GROOVE = 4, CPG_DSPRING = 5, CPG_DRSPRING = 6,
       CPG_ROTLIMIT = 7, CPG_RATCHET = 8, CPG_GEAR = 9, CPG_MOTOR = 10 };
/* arbiter states, chipmunk_structs.h:83-95 */
enum { CPG_ARB_FIRST = 0, CPG_ARB_NORMAL = 1, CPG_ARB_IGNORE = 2, CPG_ARB_CACHED = 3, CPG_ARB_INVALIDATED = 4 };
/* cpgArb.pad bit: the arbiter is held by a sleeping body, out of the cache */
#define CPG_ARB_ASLEEP 1
/* cpgArb.pad bit: the arbiter was created by this step's update (cpArbiterInit) */
#define CPG_ARB_FRESH 2
/* error bits latched in cpgTree.error */
enum { CPG_ERR_NODES = 1, CPG_ERR_PAIRS = 2, CPG_ERR_CANDS = 4, CPG_ERR_ARBS = 8, CPG_ERR_BINS = 16, CPG_ERR_LEVELS = 32, CPG_ERR_FLOW = 64,
       CPG_ERR_HASH = 128 };

/* upper bound on the blocks of the cooperative sweep-and-prune sort */
#define CPG_SORT_MAX_BLOCKS 1024

#define CPG_KEY_EMPTY 0ull
#define CPG_KEY_TOMB 1ull

/* Per-world offsets and capacities (host-written, read-only on device). */
typedef struct cpgWorld {
	int bodyOff, nbodies, ndyn;   /* dynamic+kinematic bodies are [0, ndyn) */
	int shapeOff, nshapes;
	int vertOff, nverts;          /* polygon vertex storage */
	int consOff, ncons;
	int nodeOff, nodeCap;
	int pairOff, pairCap;
	int dbinOff, dbinCap;         /* leaf-set bins of the dynamic tree */
	int sbinOff, sbinCap;         /* leaf-set bins of the static tree */
	int candOff, candCap;         /* candidate pairs emitted per step */
	int unitOff, unitCap;         /* solver units: arbiters then joints */
	int opOff, nops;              /* pending index insertions */
	int partOff;                  /* CSR of non-colliding joint partners */
	int dynShapeOff, ndynShapes;  /* shapes on non-static bodies (coloured mode) */
	int springOff;                /* CSR of the springs on each body */
} cpgWorld;

/* Per-world step parameters (host-written each step). */
typedef struct cpgParams {
	double dt, dt_coef, damping, slop, biasCoef, gx, gy;
	int iterations;
	unsigned stamp;               /* cpSpace.stamp after the increment */
	unsigned persistence;
	int active;                   /* 0: world skipped this launch */
} cpgParams;

/* Per-world device-resident tree/bookkeeping state. */
typedef struct cpgTree {
	int dynRoot, statRoot;
	unsigned treeStamp;           /* stamp of the dynamic (master) tree */
	int freeNode, nodeTop;
	int freePair, pairTop;
	unsigned dynSize, dynEntries;
	unsigned statSize, statEntries;
	int ncand;                    /* candidates emitted this step */
	int narb;                     /* arbiters in the solve list */
	int nunits;                   /* arbiters + joints */
	int nlevels;                  /* schedule depth of one sweep */
	int error;
	int pairsLive;
	int maxChain;
	int moved;                    /* leaves reinserted this step */
	/* spatial hash (a single world): bin pool tops and free lists of the
	 * dynamic and static grids, the grids' stamps (cpSpaceHash.stamp) */
	int gbinTop[2], gbinFree[2];
	unsigned gstamp[2];
} cpgTree;

/* AABB-tree node (cpBBTree.c:46-60), 96 bytes.  Each box coordinate x
 * is also kept as the pair of floats rounded down and up from it
 * (xlo <= x <= xhi), maintained by every box write in cpg_tree.cuh. */
typedef struct cpgNode {
	double l, b, r, t;
	float llo, lhi, blo, bhi, rlo, rhi, tlo, thi;
	int parent, A, B;
	int obj;                      /* shape index for leaves, -1 internal */
	unsigned stamp;
	int pairs;                    /* leaves: head of the pair thread list */
	int binNext;                  /* leaves: next leaf in the hash bin */
	int pad;
} cpgNode;

/* Cached leaf pair (cpBBTree.c:62-72), 32 bytes. */
typedef struct cpgPair {
	int aPrev, aLeaf, aNext;
	int bPrev, bLeaf, bNext;
	unsigned id;
	int pad;
} cpgPair;

/* Candidate emitted by the tree traversal, in solve-order. */
typedef struct cpgCand {
	int a, b;                     /* shapes, in the order the query passes them */
	int pair;                     /* cached pair receiving the new GJK id, or -1 */
	unsigned idIn;
} cpgCand;

/* Narrow-phase result for one candidate. */
typedef struct cpgNarrow {
	double nx, ny;
	double p1x[2], p1y[2], p2x[2], p2y[2];
	unsigned long long hash[2];
	int count;                    /* 0..2 contacts */
	int flip;                     /* 1 when info.a is the candidate's b */
	unsigned idOut;
	int pad;
} cpgNarrow;

typedef struct cpgContact {
	double r1x, r1y, r2x, r2y;
	double nMass, tMass, bounce, jnAcc, jtAcc, jBias, bias;
	unsigned long long hash;
} cpgContact;

/* Cached arbiter (chipmunk_structs.h:124-145), one per table slot. */
typedef struct cpgArb {
	int a, b;                     /* shapes, info order of the last update */
	int ba, bb;                   /* their bodies */
	int count, state;
	unsigned stamp;
	int world;
	unsigned gjk;                 /* last GJK feature id of the pair */
	int colorTag;                 /* coloured mode: valid bit, low 23 bits of the colouring step's stamp, colour */
	int warmSrc;                  /* per contact k, bits 4k..4k+3: 1 + index of the old contact whose impulses it took (0: none) */
	int pad;
	double nx, ny, e, u, svx, svy;
	cpgContact c[2];
} cpgArb;

/* Joint (cpPivotJoint/cpPinJoint/cpSlideJoint), one record per joint. */
typedef struct cpgJoint {
	int kind, a, b, colorTag;     /* colorTag: as in cpgArb */
	double ax, ay, bx, by;        /* anchors in body space */
	double maxForce, biasCoef, maxBias;
	double dist, min, max;
	double r1x, r1y, r2x, r2y;
	double k11, k12, k21, k22;    /* pivot: inverse mass tensor */
	double jx, jy;                /* pivot: accumulated impulse */
	double biasx, biasy;          /* pivot: bias velocity */
	double nx, ny, nMass, jnAcc, bias;  /* pin/slide; nMass holds iSum and bias the
	                                     * spring's target velocity for the other kinds */
	double gax, gay, gbx, gby, gnx, gny; /* groove: ends and normal in body a's space */
	double restLength, stiffness, damping; /* springs (rotary spring: restLength is the rest angle) */
	double phase, ratchet, angle, ratio, ratioInv, rate; /* ratchet, gear, motor */
	double coef, clamp;                  /* spring damping coefficient, groove clamp (pre-step) */
	double preJx, preJy;                 /* the springs' pre-step impulse (rotary: preJx) */
} cpgJoint;

/* Solver rows: one per unit, stored in schedule order so that the threads
 * of one level read consecutive rows.  Built by the pre-step, consumed by
 * the warm start and the iterations, written back to the arbiters and
 * joints at the end of the solve. */
typedef struct cpgRowContact {
	double r1x, r1y, r2x, r2y;
	double nMass, tMass, bounce, bias;
	double jnAcc, jtAcc, jBias, pad;
} cpgRowContact;

typedef struct cpgRow {
	int a, b;                     /* world-local bodies */
	int kind;                     /* 0: arbiter, else CPG_PIVOT/PIN/SLIDE */
	int count;                    /* arbiter contacts */
	int src;                      /* arbiter slot, or joint index in the world */
	int flags;                    /* 1: first step (no warm start); 2/4: body a/b dynamic */
	union {
		struct { double nx, ny, u, svx, svy, e; cpgRowContact c[2]; } arb;   /* e: elasticity */
		struct { double r1x, r1y, r2x, r2y, k11, k12, k21, k22, jx, jy, biasx, biasy;
		         double nx, ny, nMass, jnAcc, bias, maxForce;
		         double clamp, coef, aux1, aux2; } jnt;   /* groove clamp; spring coefficient; ratchet / gear ratios */
	};
} cpgRow;

/* Pending index edit, replayed on the device in call order before the
 * next step.  An insertion (cpSpaceAddShape, cpBodySetType) carries the
 * shape's box and its body's velocity as they were at that call (the
 * reference builds the leaf's fattened box immediately,
 * cpBBTree.c:605-616); a removal (cpSpaceRemoveShape, cpBodySetType)
 * names the shape and the index it leaves (cpBBTree.c:619-630). */
enum { CPG_OP_INSERT = 0, CPG_OP_REMOVE = 1, CPG_OP_REINDEX = 2, CPG_OP_REINDEX_STATIC = 3, CPG_OP_USE_HASH = 4 };
/* CPG_OP_REINDEX (cpSpaceReindexShape) carries the shape's new cached box
 * and its body's velocity; CPG_OP_REINDEX_STATIC (cpSpaceReindexStatic)
 * re-indexes every static leaf against the shapes' uploaded boxes. */
typedef struct cpgOp {
	int shape;
	int isStatic;
	int kind;                     /* CPG_OP_INSERT or CPG_OP_REMOVE */
	int pad1;
	double l, b, r, t;
	double vx, vy;
} cpgOp;

/* A spatial query (cpSpaceQuery.c) and one of its results. */
enum { CPG_Q_POINT = 0, CPG_Q_POINT_NEAREST = 1, CPG_Q_SEGMENT = 2, CPG_Q_SEGMENT_FIRST = 3, CPG_Q_BB = 4,
       CPG_Q_SHAPE_POINT = 5, CPG_Q_SHAPE_SEGMENT = 6 };   /* the last two: one shape, slot in pad */
typedef struct cpgQuery {
	double ax, ay, bx, by;        /* point | segment start, end | box l, b, r, t */
	double r;                     /* maximum distance | segment radius */
	unsigned long long group;     /* the query's cpShapeFilter */
	unsigned cat, mask;
	int kind;
	int pad;
} cpgQuery;
/* A shape given to a shape query or to cpShapesCollide by value: its
 * world-space cache (circle tc | segment ta, tb, tn; polygon planes at
 * voff of the query's plane array), the segment tangents in body space,
 * its body's rotation, box, filter and sensor flag; slot is its place in
 * the queried world, -1 when it is not one of its shapes. */
typedef struct cpgProbe {
	double r, p0x, p0y, p1x, p1y, nx, ny, atx, aty, btx, bty, rotx, roty;
	double bbl, bbb, bbr, bbt;
	unsigned long long hashid, group;
	unsigned cat, mask;
	int kind, count, voff, slot, sensor, pad;
} cpgProbe;
/* One shape found by a shape query, with its contact point set
 * (cpShape.c:258-283). */
typedef struct cpgShapeHit {
	int shape, count, sensor, pad;
	double nx, ny;
	double ax[2], ay[2], bx[2], by[2], dist[2];
} cpgShapeHit;

typedef struct cpgHit {
	int shape;                    /* world-local shape slot, -1 none */
	int pad;
	double px, py;                /* point */
	double d;                     /* distance | alpha */
	double gx, gy;                /* gradient | normal */
} cpgHit;

/* All device arrays of a set.  Vectors are split into x/y arrays. */
/* Recording of replayed steps for the differentiable rollout. */
#define CPG_PAIR_TYPES 6

/* Reverse solve: doubles of a contact lane's scratch (AdjLaneBar), block
 * size, and the largest world whose body adjoints it keeps in shared memory. */
#define CPG_ADJ_LANE_DOUBLES 12
#define CPG_ADJ_SOLVE_THREADS 64
#define CPG_ADJ_STAGED_BODIES 1024

/* What a rollout records of one segment of K steps.  The forward fills
 * everything but `app` (the light tape); the solver's per-iteration records
 * are recomputed from it by the reverse pass, or recorded together with the
 * rest when a segment is replayed from its checkpoint. */
typedef struct cpgTape {
	int on;                   /* record this step */
	int step;                 /* its index within the segment */
	int K;                    /* steps per segment */
	int rowCap, levCap;
	double *body;             /* [K][8][totalBodies] planes: p.x p.y a (after position integration), v.x v.y w (pre-step), cos, sin */
	double *vel;              /* [K][3][totalBodies] planes: v.x v.y w after velocity integration (the solve's input) */
	double *shape;            /* [K][6][totalShapes] planes: world p0.x p0.y p1.x p1.y n.x n.y */
	double *verts;            /* [K][4][totalVerts] planes: world vertex x y, world normal x y */
	cpgParams *params;        /* [K][nworlds] */
	cpgRow *rows;             /* [rowCap] rows of all recorded steps, world by world */
	int *rowInfo;             /* [rowCap][4]: arbiter shapes a, b; final GJK id; warm-start sources */
	int *rowWorld;            /* [rowCap] world of the row */
	int *rowOff;              /* [K][nworlds + 1] */
	int *levels;              /* [levCap] level starts (relative to the world's rows) */
	int *levOff;              /* [K][nworlds + 1] */
	double *app;              /* [rowCap][iterations][2] impulse application records (AdjApp); NULL: not recorded */
	int *cursor;              /* [4]: rows used, levels used, overflow flag, unsupported-row flag */
} cpgTape;

typedef struct cpgSet {
	int nworlds;
	int totalBodies, totalShapes, totalVerts, totalCons;
	int totalNodes, totalPairs, totalDBins, totalSBins, totalCands, totalUnits, totalOps, totalParts, totalSprings;
	int arbCap;                   /* arbiter hash table slots (power of two) */
	int maxWorldUnits;

	cpgWorld *world;              /* [nworlds] */
	cpgParams *params;            /* [nworlds] */
	cpgTree *tree;                /* [nworlds] */

	/* bodies [totalBodies] */
	double *px, *py, *vx, *vy, *fx, *fy, *ang, *w, *tq;
	double *ta, *tb, *tc, *td, *ttx, *tty;   /* transform */
	double *vbx, *vby, *wb;
	double *m, *minv, *i, *iinv, *cogx, *cogy;
	int *btype, *bworld;
	int *partStart, *partCount;   /* joint partners with collideBodies off */
	int *parts;                   /* [totalParts] */
	int *springStart, *springCount; /* damped springs (linear and rotary) on each body, */
	int *springs;                 /* [totalSprings] their world-local joint indices in constraint order */
	int *last;                    /* schedule scratch */

	/* shapes [totalShapes] */
	int *skind, *sbody, *sleaf, *sworld, *svoff, *svcount;
	double *sr;
	double *s0x, *s0y, *s1x, *s1y, *snx, *sny;   /* local: circle c | seg a, b, n */
	double *w0x, *w0y, *w1x, *w1y, *wnx, *wny;   /* world: circle tc | seg ta, tb, tn */
	double *atx, *aty, *btx, *bty;               /* segment tangents */
	double *bbl, *bbb, *bbr, *bbt;
	double *se, *su, *svx, *svy;
	unsigned long long *sgroup;
	unsigned *scat, *smask;
	unsigned char *ssensor;
	unsigned char *shost;         /* 1: the shape's collision type has a handler (its arbiters go to the host) */
	unsigned long long *shash;    /* cpShape.hashid */

	/* polygon planes [totalVerts]: local and world */
	double *lvx, *lvy, *lnx, *lny, *gvx, *gvy, *gnx, *gny;

	/* tree */
	cpgNode *nodes;               /* [totalNodes] */
	cpgPair *pairs;               /* [totalPairs] */
	int *dbins, *sbins;
	cpgOp *ops;                   /* [totalOps] */

	/* per-step collision data [totalCands] */
	cpgCand *cands;
	cpgNarrow *narrow;
	/* narrow-phase scratch outside the slab: candidates that pass
	 * QueryReject, by pair type ([CPG_PAIR_TYPES][totalCands] flat
	 * candidate indices), and the per-type counts */
	int *nbucket;
	int *nbCount;
	int *candArb;                 /* arbiter slot pushed to the solve list, or -1 */
	int *arbList;                 /* solve list: arbiter slots, per world */
	int *prevList;                /* previous step's solve list */
	int *prevCount;               /* [nworlds] */

	/* arbiter hash table [arbCap] */
	unsigned long long *keys;
	cpgArb *arbs;

	/* joints [totalCons] */
	cpgJoint *joints;
	double *jbias;                /* 1 - pow(errorBias, dt), host-computed */

	/* solver rows [totalUnits] and packed body state [totalBodies*8]:
	 * vx vy w vbx vby wb minv iinv */
	cpgRow *rows;
	double *pbody;

	/* schedule [totalUnits] */
	int *unitA, *unitB;           /* dynamic bodies touched (-1 none) */
	int *unitKey;                 /* coloured mode: deterministic unit id */
	int *worldOrder;              /* [nworlds] worlds by decreasing size */
	int *unitLevel, *unitOrder;
	int *levelStart;              /* [totalUnits + nworlds] */

	/* coloured mode (single-world sets) */
	int *dynShapes;               /* [totalShapes] shapes on non-static bodies */
	unsigned *sortKA, *sortKB, *rkeys, *sapCount, *rsHist;   /* rsHist: [256*CPG_SORT_MAX_BLOCKS + 256] */
	unsigned long long *sortK64;  /* [totalShapes] (key << 32 | shape) in the previous sweep order */
	int *sortVA, *sortVB;
	unsigned long long *claim, *cmask;   /* [totalBodies] */
	int *colorCursor;             /* [512]: [0..1] colouring round counters, [8] sweep axis, [10] n+1 once a sweep order exists, [11] its axis, [12] dataflow wait gave up, [13] no dataflow this step (a colour past 63), [16..31] transposition swap counters, [256..511] colour counts */
	long long *sapBB;             /* [4*totalShapes] box keys in sweep order */
	/* dataflow sweep of the coloured mode: each unit waits for the units
	 * before it on its two bodies instead of a grid barrier per colour */
	int *flowPred;                /* [2*totalUnits] per unit (schedule position) and body: predecessor position << 1 | previous pass, -1 none */
	int *flowDone;                /* [totalUnits] passes the unit has finished */
	int *flowPos;                 /* [64*totalBodies] schedule position of the unit of colour c on body b */
	int flowSolve;                /* 1: coloured solve by dataflow (host value) */
	int flowSpin;                 /* polls before a dataflow wait gives up; 0: the default (host value) */
	int flowWithhold;             /* test of the wait limit: completions are not published (host value) */
	int warmGather;               /* 1: coloured mode applies the cached impulses per body in k_integrate_vel (host value) */
	int parMark;                  /* 1: a single world's tree is marked by k_tree_mark's parallel phases (host value) */
	int hostCoopBlocks;           /* > 0: at most this many blocks in the cooperative kernels (host value) */
	int bridge;                   /* 1: collision handlers run on the host (a single world): k_arb_update lists every
	                                 colliding arbiter and leaves the sensor/ignore rule to the host (host value) */
	int *sepSlots, *sepCount;     /* bridge: slots of the arbiters the cache filter separates this step */
	/* spatial hash (cpSpaceUseSpatialHash, a single world): the handle sets
	 * are the leaf sets, the handles nodes; cells of the dynamic then the
	 * static grid, and a bin pool for each (gbinCap bins each) */
	int useHash, numcells, gbinCap;
	double celldim;
	int *gcells, *gbinHandle, *gbinNext;
	int *markScratch;             /* single-world sets: the parallel marking's scratch (mark_scratch in cpg_kernels.cu) */
	float *sapPart;               /* [4*CPG_SORT_MAX_BLOCKS] per-block centre sums for the sweep axis */
	int hostNdyn;                 /* dynamic shapes of world 0 (host value) */
	int hostUnitsHint;            /* solver units of world 0 last step (host value) */
	int hostMaxBodies;            /* largest world (host value) */
	int hostMaxNodes;             /* largest world's node pool (host value) */
	int hostTreeStage;            /* worlds of at most this many nodes run the tree from shared memory; -1: all that fit */
	int hostSolveThreads;         /* block size of the per-world solve; 0: default */
	int hostSolveStage;           /* worlds of at most this many bodies solve from shared memory; -1: all that fit */
	int solveLayout;              /* per-level lane layout: 0 automatic, 1 fewest instructions, 2 shortest chain, 3 four lanes only */

	/* stats block copied to the host after each step */
	int *stats;

	/* differentiable rollout: recording of a replayed step (on = 0 otherwise) */
	cpgTape tape;
} cpgSet;

/* Adjoint state of the differentiable rollout (device arrays). */
typedef struct cpgAdj {
	double *body;                 /* [totalBodies][9]: adjoints of p.x p.y a v.x v.y w v_bias.x v_bias.y w_bias */
	double *arb;                  /* [arbCap][2][2]: adjoints of the stored jnAcc, jtAcc of each arbiter contact */
	double *gMinv;                /* [totalBodies] dL/d(1/m) */
	double *gE, *gU;              /* [totalShapes] dL/de, dL/du */
	double *con;                  /* [rows of one step][2][4][CPG_ADJ_LANE_DOUBLES] per contact and lane scratch */
	double *unit;                 /* [rows of one step][20] per-unit contributions of the pre-step and geometry adjoints */
	double *arbTmp;               /* [arbCap][2][2] remapping buffer */
	cpgRow *srows;                /* [rows of one segment] rows the recomputed solves run on */
	double *sbodies;              /* [K][totalBodies][8] packed bodies of the recomputed solves (worlds too large for shared memory) */
} cpgAdj;

/* ---- launchers (cpg_kernels.cu) ---- */
int cpg_launch_apply_ops(const cpgSet *s, void *stream);
int cpg_launch_step(const cpgSet *s, const cpgSet *host_mirror, int mode, void *stream, float *phase_ms);
int cpg_launch_gather_arbs(const cpgSet *s, int world, cpgArb *out, int n, void *stream);
int cpg_launch_step_part(const cpgSet *s, const cpgSet *h, int mode, void *stream, float *phase_ms, int part);
int cpg_launch_gather_slots(const cpgSet *s, const int *slots, cpgArb *out, int n, void *stream);
int cpg_launch_gather_pairs(const cpgSet *s, int world, int *out, int n, void *stream);
int cpg_launch_gather_keys(const cpgSet *s, const unsigned long long *keys, cpgArb *out, int n, void *stream);
int cpg_launch_put_arbs(const cpgSet *s, const int *slots, const cpgArb *recs, int n, void *stream);
int cpg_launch_shape_arbs(const cpgSet *s, int shape, int *slots, int *count, int cap, void *stream);
int cpg_launch_sleep_edits(const cpgSet *s, const unsigned long long *keys, const int *ops, const unsigned *stamps, int n,
                           const unsigned long long *listKeys, int nlist, void *stream);
long long cpg_launch_count(int reset);
int cpg_launch_tape(const cpgSet *s, void *stream);
int cpg_launch_adjoint(const cpgSet *s, const cpgAdj *a, int step, int rows, void *stream);
int cpg_launch_adjoint_remap(const cpgSet *s, const cpgAdj *a, const void *oldKeys, void *stream);
int cpg_launch_tape_vel(const cpgSet *s, void *stream);
int cpg_launch_step_graph(const cpgSet *s, int mode, void *stream, void **cache);
void cpg_step_graph_free(void *cache);
int cpg_launch_replay_solve(const cpgSet *s, const cpgAdj *a, int nsteps, void *stream);
int cpg_launch_transfer(const cpgSet *to, const cpgSet *from, const int *bodyMap, const unsigned char *deadShape,
                        int *slotMap, void *stream);
int cpg_launch_contact_quality(const cpgSet *s, int w, double dt, double *acc, void *stream);
int cpg_launch_body_states(const cpgSet *s, int w, double *out, int n, void *stream);
int cpg_launch_shape_query(const cpgSet *s, int world, const cpgProbe *probe, const double *planes, int nplanes,
                           int brute, cpgShapeHit *hits, int cap, int *counts, void *stream);
int cpg_launch_shape_pair(const cpgProbe *probes, const double *planes, int nplanes, cpgShapeHit *hit,
                          int *counts, void *stream);
int cpg_launch_query(const cpgSet *s, int world, const cpgQuery *queries, int nq, cpgHit *hits, int cap,
                     int *counts, int brute, int *status, void *stream);
int cpg_launch_set_arb_impulses(const cpgSet *s, int w, const double *imp, const int *pairs, int n, int *mismatch, void *stream);

#ifdef __cplusplus
}
#endif

#endif

/*
 * cp_oracle.c -- CPU restatement of Chipmunk2D 7.0.3's cpSpaceStep path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: the tests, the
 * smoke check and the CPU-baseline leg of bench.py load it (as
 * liboracle.so) to check and time the GPU library.  The GPU library never
 * links, loads or calls it.
 *
 * It restates, in plain C with index-based containers, every stage the GPU
 * path implements: body integration, shape caches, the incremental AABB tree
 * with its per-leaf pair cache (which fixes the order arbiters are solved
 * in), the six narrow-phase routines with GJK/EPA, the arbiter cache with
 * warm starting, and the sequential-impulse solver with pivot, pin and slide
 * joints.  Floating-point expressions keep the reference's operation order,
 * because bit-for-bit agreement is the point; the oracle is pinned against
 * the compiled reference (oracle/build_ref.sh) by tests/test_oracle_ref.py,
 * and against committed fixtures by tests/test_oracle_golden.py.
 *
 * Every function cites the reference file:line it follows.  Build with
 * -ffp-contract=off and without -ffast-math (oracle/build_oracle.sh).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdarg.h>
#include <pthread.h>
#include "../include/chipmunk_gb300.h"

#define ORC_INF ((cpFloat)INFINITY)

/* ========================================================================
 * Errors: include/chipmunk/chipmunk.h:50-58, src/chipmunk.c:31-54
 * ====================================================================== */
const char *cpVersionString = "7.0.3";

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

#define ORC_ASSERT(cond, msg) do { if(!(cond)){ cpMessage(#cond, __FILE__, __LINE__, 1, 1, msg); abort(); } } while(0)

/* ========================================================================
 * Scalar helpers: chipmunk_types.h:137-168 (cpfmax/cpfmin use a > b / a < b,
 * not fmax/fmin -- NaN handling differs).
 * ====================================================================== */
static inline cpFloat fmax_(cpFloat a, cpFloat b) { return (a > b) ? a : b; }
static inline cpFloat fmin_(cpFloat a, cpFloat b) { return (a < b) ? a : b; }
static inline cpFloat fabs_(cpFloat f) { return (f < 0) ? -f : f; }
static inline cpFloat fclamp_(cpFloat f, cpFloat lo, cpFloat hi) { return fmin_(fmax_(f, lo), hi); }
static inline cpFloat fclamp01_(cpFloat f) { return fmax_(0.0, fmin_(f, 1.0)); }
static inline cpVect vclamp_(cpVect v, cpFloat len) { return (cpvdot(v, v) > len*len) ? cpvmult(cpvnormalize(v), len) : v; }
static inline cpBB bbmerge_(cpBB a, cpBB b) { return cpBBNew(fmin_(a.l, b.l), fmin_(a.b, b.b), fmax_(a.r, b.r), fmax_(a.t, b.t)); }
static inline cpFloat bbmergedarea_(cpBB a, cpBB b) { return (fmax_(a.r, b.r) - fmin_(a.l, b.l))*(fmax_(a.t, b.t) - fmin_(a.b, b.b)); }
static inline cpFloat bbproximity_(cpBB a, cpBB b) { return fabs_(a.l + a.r - b.l - b.r) + fabs_(a.b + a.t - b.b - b.t); }
static inline cpTransform rigid_inverse_(cpTransform t)
{
	return cpTransformNewTranspose(t.d, -t.c, (t.c*t.ty - t.tx*t.d), -t.b, t.a, (t.tx*t.b - t.a*t.ty));
}
static inline cpVect mat2_mul_(cpMat2x2 m, cpVect v) { return cpv(v.x*m.a + v.y*m.b, v.x*m.c + v.y*m.d); }

#define HASH_COEF ((cpHashValue)3344921057ul)
#define HASH_PAIR(A, B) ((cpHashValue)(A)*HASH_COEF ^ (cpHashValue)(B)*HASH_COEF)

/* ========================================================================
 * Object layouts (oracle-private)
 * ====================================================================== */
enum { SHAPE_CIRCLE = 0, SHAPE_SEGMENT = 1, SHAPE_POLY = 2 };
enum { JOINT_PIVOT = 1, JOINT_PIN = 2, JOINT_SLIDE = 3, JOINT_GROOVE = 4, JOINT_DSPRING = 5, JOINT_DRSPRING = 6,
       JOINT_ROTLIMIT = 7, JOINT_RATCHET = 8, JOINT_GEAR = 9, JOINT_MOTOR = 10 };
enum { ARB_FIRST = 0, ARB_NORMAL = 1, ARB_IGNORE = 2, ARB_CACHED = 3, ARB_INVALID = 4 };

typedef struct Contact {
	cpVect r1, r2;
	cpFloat nMass, tMass, bounce, jnAcc, jtAcc, jBias, bias;
	cpHashValue hash;
} Contact;

struct cpArbiter {
	cpFloat e, u;
	cpVect surface_vr;
	cpShape *a, *b;
	cpBody *body_a, *body_b;
	int count;
	Contact contacts[2];
	cpVect n;
	cpBool swapped;
	cpTimestamp stamp;
	int state;
	int live;   /* slot in use in the cache */
	/* the contact graph (cpArbiterThread, chipmunk_structs.h:176-179):
	 * body_a's and body_b's list links, as slot + 1 (0 = none) */
	int prevA, nextA, prevB, nextB;
	/* collision handlers of the last update (chipmunk_structs.h:210-214) */
	cpCollisionHandler *handler, *handlerA, *handlerB;
	cpDataPointer data;
};

struct cpBody {
	cpBodyVelocityFunc velocity_func;
	cpBodyPositionFunc position_func;
	cpFloat m, m_inv, i, i_inv;
	cpVect cog, p, v, f;
	cpFloat a, w, t;
	cpTransform transform;
	cpDataPointer userData;
	cpVect v_bias;
	cpFloat w_bias;
	cpSpace *space;
	cpShape *shapeList;
	cpConstraint *constraintList;
	cpFloat idleTime;
	/* sleeping (chipmunk_structs.h:90-94): the component root and next
	 * body; the head of the body's arbiter list, as slot + 1 (0 = none) */
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
	cpCollisionType type;
	cpShapeFilter filter;
	cpShape *next, *prev;
	cpHashValue hashid;
	int leaf;            /* tree node index, -1 when not indexed */
	/* circle */
	cpVect c, tc;
	cpFloat r;           /* circle, segment and poly radius */
	/* segment */
	cpVect sa, sb, sn, ta, tb, tn, a_tangent, b_tangent;
	/* poly: world planes [0,count), local planes [count,2count) */
	int count;
	cpVect *pv;          /* plane points, 2*count */
	cpVect *pn;          /* plane normals, 2*count */
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
	cpFloat dist, min, max;     /* pin: dist; slide: min/max */
	cpVect r1, r2;
	cpMat2x2 k;                 /* pivot */
	cpVect jAcc, biasv;         /* pivot */
	cpVect n;                   /* pin, slide, damped spring */
	cpFloat nMass, jnAcc, bias; /* pin, slide; jnAcc is the scalar jAcc of the other kinds */
	/* groove (chipmunk_structs.h:307-318) */
	cpVect grv_n, grv_a, grv_b, grv_tn;
	cpFloat clamp;
	/* springs (chipmunk_structs.h:320-345) */
	cpFloat restLength, stiffness, damping, target_vrn, v_coef;
	cpFloat restAngle, target_wrn, w_coef;
	cpDampedSpringForceFunc springForceFunc;
	cpDampedRotarySpringTorqueFunc springTorqueFunc;
	/* rotary limit, ratchet, gear, motor (chipmunk_structs.h:347-385) */
	cpFloat iSum, angle, phase, ratchet, ratio, ratio_inv, rate;
};

/* ---- AABB tree: index-based nodes and pairs (src/cpBBTree.c:32-72) ---- */
typedef struct Node {
	cpShape *obj;        /* NULL for internal nodes */
	cpBB bb;
	int parent;
	int A, B;            /* children of internal nodes */
	cpTimestamp stamp;   /* leaves */
	int pairs;           /* leaves: head of the pair list */
	int binNext;         /* leaves: chain in the leaf hash set */
} Node;

typedef struct Thread { int prev, leaf, next; } Thread;
typedef struct Pair { Thread a, b; cpCollisionID id; } Pair;

/* Leaf set with the reference's table behaviour (src/cpHashSet.c:87-253):
 * prime-sized bins, head insertion, rehash on entries >= size.  Only the
 * iteration order matters here: leaves are re-indexed in bin order. */
typedef struct LeafSet {
	unsigned int size, entries;
	int *bins;
} LeafSet;

typedef struct Tree {
	int root;
	LeafSet leaves;
	int isDynamic;       /* dynamic tree: fattened boxes, owns the stamp */
} Tree;

/* The cells of a spatial hash (src/cpSpaceHash.c:28-43, 99-115): each cell
 * a list of bins (head insertion) naming a handle.  A handle is a node of
 * the index's pool whose leaf set is the hash's handle set; its stamp is
 * the handle's stamp. */
typedef struct HashGrid {
	int numcells;
	cpFloat celldim;
	int *cells;                          /* first bin of each cell, -1 */
	int *binHandle, *binNext; int nbins, capbins, freeBin;
	cpTimestamp stamp;
} HashGrid;

typedef struct ArbMap {
	int cap;             /* power of two */
	int used;            /* live + tombstones */
	uint64_t *keys;      /* 0 = empty, 1 = tombstone */
	int *slot;
} ArbMap;

struct cpSpace {
	int iterations;
	cpVect gravity;
	cpFloat damping, idleSpeedThreshold, sleepTimeThreshold;
	cpFloat collisionSlop, collisionBias;
	cpTimestamp collisionPersistence;
	cpDataPointer userData;
	cpTimestamp stamp;
	cpFloat curr_dt;
	int locked;
	cpHashValue shapeIDCounter;

	cpBody **dyn; int ndyn, capdyn;
	cpBody **stat; int nstat, capstat;
	cpConstraint **cons; int ncons, capcons;

	/* index */
	Node *nodes; int nnodes, capnodes, freeNode;
	Pair *pairs; int npairs, cappairs, freePair;
	Tree dynTree, statTree;
	cpTimestamp treeStamp;
	/* cpSpaceUseSpatialHash: both indices are spatial hashes; the trees'
	 * leaf sets are the handle sets */
	int useHash;
	HashGrid dynGrid, statGrid;

	/* pairs that passed the box test in the last step (for broadphase checks) */
	int *candPairs; int ncand, capcand;

	/* arbiters */
	cpArbiter *arbs; int narbs, caparbs, freeArb;
	int *freeList; int nfree, capfree;
	ArbMap amap;
	int *active; int nactive, capactive;   /* space->arbiters: slot indices */

	/* collision handlers (cpSpace.c:65-103, 378-413): the default one and
	 * the registered ones, each on the heap */
	cpCollisionHandler defaultHandler;
	int usesWildcards;
	cpCollisionHandler **handlers; int nhandlers, caphandlers;

	/* sleeping components (their roots) and bodies woken while locked */
	cpBody **sleeping; int nsleeping, capsleeping;
	cpBody **roused; int nroused, caproused;

	cpBody staticBody;
	struct Hasty *hasty;                   /* the threaded solver (cpx_space_set_hasty), or NULL */
	struct PostStep *post; int npost, cappost, postRunning;   /* post-step callbacks */
};

static void run_post_step_(cpSpace *sp);
static void arb_unthread_(cpSpace *sp, int slot);
static void space_unlock_(cpSpace *sp);

/* cpConstraintActivateBodies (chipmunk_private.h:165-170) */
static void activate_bodies_(cpConstraint *c) { cpBodyActivate(c->a); cpBodyActivate(c->b); }

/* ========================================================================
 * Creation-time math: src/chipmunk.c:63-171, 250-274
 * ====================================================================== */
cpFloat cpMomentForCircle(cpFloat m, cpFloat r1, cpFloat r2, cpVect offset)
{
	return m*(0.5*(r1*r1 + r2*r2) + cpvlengthsq(offset));
}

cpFloat cpAreaForCircle(cpFloat r1, cpFloat r2)
{
	return (cpFloat)3.14159265358979323846264338327950288*fabs_(r1*r1 - r2*r2);
}

cpFloat cpMomentForSegment(cpFloat m, cpVect a, cpVect b, cpFloat r)
{
	cpVect offset = cpvlerp(a, b, 0.5);
	cpFloat length = cpvdist(b, a) + 2.0*r;
	return m*((length*length + 4.0*r*r)/12.0 + cpvlengthsq(offset));
}

cpFloat cpAreaForSegment(cpVect a, cpVect b, cpFloat r)
{
	return r*((cpFloat)3.14159265358979323846264338327950288*r + 2.0*cpvdist(a, b));
}

cpFloat cpMomentForPoly(cpFloat m, int count, const cpVect *verts, cpVect offset, cpFloat r)
{
	(void)r;
	if(count == 2) return cpMomentForSegment(m, verts[0], verts[1], 0.0);
	cpFloat sum1 = 0.0, sum2 = 0.0;
	for(int i = 0; i < count; i++){
		cpVect v1 = cpvadd(verts[i], offset);
		cpVect v2 = cpvadd(verts[(i + 1)%count], offset);
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
	return r*((cpFloat)3.14159265358979323846264338327950288*fabs_(r) + perimeter) + area/2.0;
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

cpFloat cpMomentForBox(cpFloat m, cpFloat width, cpFloat height)
{
	return m*(width*width + height*height)/12.0;
}

cpFloat cpMomentForBox2(cpFloat m, cpBB box)
{
	cpFloat width = box.r - box.l, height = box.t - box.b;
	cpVect offset = cpvmult(cpv(box.l + box.r, box.b + box.t), 0.5);
	return cpMomentForBox(m, width, height) + m*cpvlengthsq(offset);
}

/* QuickHull with in-place partitioning (src/chipmunk.c:178-274).  The
 * output vertex order feeds contact feature ids, so the partition steps
 * follow the reference exactly. */
static void hull_extremes(const cpVect *verts, int count, int *start, int *end)
{
	*start = *end = 0;
	cpVect lo = verts[0], hi = lo;
	for(int i = 1; i < count; i++){
		cpVect v = verts[i];
		if(v.x < lo.x || (v.x == lo.x && v.y < lo.y)){
			lo = v; *start = i;
		} else if(v.x > hi.x || (v.x == hi.x && v.y > hi.y)){
			hi = v; *end = i;
		}
	}
}

static inline void vswap(cpVect *a, cpVect *b) { cpVect t = *a; *a = *b; *b = t; }

static int hull_partition(cpVect *verts, int count, cpVect a, cpVect b, cpFloat tol)
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
			vswap(&verts[head], &verts[tail]);
			tail--;
		}
	}
	if(pivot != 0) vswap(&verts[0], &verts[pivot]);
	return head;
}

static int hull_reduce(cpFloat tol, cpVect *verts, int count, cpVect a, cpVect pivot, cpVect b, cpVect *result)
{
	if(count < 0) return 0;
	if(count == 0){ result[0] = pivot; return 1; }
	int left = hull_partition(verts, count, a, pivot, tol);
	int index = hull_reduce(tol, verts + 1, left - 1, a, verts[0], pivot, result);
	result[index++] = pivot;
	int right = hull_partition(verts + left, count - left, pivot, b, tol);
	return index + hull_reduce(tol, verts + left + 1, right - 1, pivot, verts[left], b, result + index);
}

int cpConvexHull(int count, const cpVect *verts, cpVect *result, int *first, cpFloat tol)
{
	if(verts != result) memcpy(result, verts, (size_t)count*sizeof(cpVect));
	int start, end;
	hull_extremes(verts, count, &start, &end);
	if(start == end){
		if(first) *first = 0;
		return 1;
	}
	vswap(&result[0], &result[start]);
	vswap(&result[1], &result[end == 0 ? start : end]);
	cpVect a = result[0], b = result[1];
	if(first) *first = start;
	return hull_reduce(tol, result + 2, count - 2, a, b, a, result + 1) + 1;
}

/* ========================================================================
 * Bodies: src/cpBody.c
 * ====================================================================== */
static cpBodyType body_type(const cpBody *b)
{
	/* cpBody.c:136-146 */
	if(b->idleTime == ORC_INF) return CP_BODY_TYPE_STATIC;
	if(b->m == ORC_INF) return CP_BODY_TYPE_KINEMATIC;
	return CP_BODY_TYPE_DYNAMIC;
}

/* cpBody.c:347-357 */
static void body_set_transform(cpBody *body, cpVect p, cpFloat a)
{
	cpVect rot = cpvforangle(a);
	cpVect c = body->cog;
	body->transform = cpTransformNewTranspose(
		rot.x, -rot.y, p.x - (c.x*rot.x - c.y*rot.y),
		rot.y,  rot.x, p.y - (c.x*rot.y + c.y*rot.x));
}

void cpBodyUpdateVelocity(cpBody *body, cpVect gravity, cpFloat damping, cpFloat dt);
void cpBodyUpdatePosition(cpBody *body, cpFloat dt);

static void body_init(cpBody *body, cpFloat mass, cpFloat moment)
{
	/* cpBody.c:33-66 */
	memset(body, 0, sizeof(*body));
	body->velocity_func = cpBodyUpdateVelocity;
	body->position_func = cpBodyUpdatePosition;
	body->m = mass;
	body->m_inv = (mass == 0.0 ? ORC_INF : 1.0/mass);
	body->i = moment;
	body->i_inv = (moment == 0.0 ? ORC_INF : 1.0/moment);
	body->a = 0.0;
	body_set_transform(body, body->p, 0.0);
}

static void body_make_static(cpBody *body)
{
	/* cpBody.c:148-167 */
	body->idleTime = ORC_INF;
	body->m = body->i = ORC_INF;
	body->m_inv = body->i_inv = 0.0;
	body->v = cpvzero;
	body->w = 0.0;
}

cpBody *cpBodyNew(cpFloat mass, cpFloat moment)
{
	ORC_ASSERT(0.0 <= mass && mass < ORC_INF, "Mass must be positive and finite.");
	ORC_ASSERT(moment >= 0.0, "Moment of Inertia must be positive.");
	cpBody *body = (cpBody *)calloc(1, sizeof(cpBody));
	body_init(body, mass, moment);
	return body;
}

cpBody *cpBodyNewStatic(void) { cpBody *b = cpBodyNew(0.0, 0.0); body_make_static(b); return b; }

cpBody *cpBodyNewKinematic(void)
{
	cpBody *b = cpBodyNew(0.0, 0.0);
	b->idleTime = 0.0;
	b->m = b->i = ORC_INF;
	b->m_inv = b->i_inv = 0.0;
	b->v = cpvzero; b->w = 0.0;
	return b;
}

void cpBodyFree(cpBody *body) { free(body); }
cpBool cpBodyIsSleeping(const cpBody *body) { return body->sleepRoot != NULL; }
cpBodyType cpBodyGetType(cpBody *body) { return body_type(body); }
cpSpace *cpBodyGetSpace(const cpBody *body) { return body->space; }
cpFloat cpBodyGetMass(const cpBody *body) { return body->m; }
void cpBodySetMass(cpBody *body, cpFloat mass) { cpBodyActivate(body); body->m = mass; body->m_inv = (mass == 0.0 ? ORC_INF : 1.0/mass); }
cpFloat cpBodyGetMoment(const cpBody *body) { return body->i; }
void cpBodySetMoment(cpBody *body, cpFloat i) { cpBodyActivate(body); body->i = i; body->i_inv = (i == 0.0 ? ORC_INF : 1.0/i); }
cpVect cpBodyGetRotation(const cpBody *body) { return cpv(body->transform.a, body->transform.b); }
cpVect cpBodyGetPosition(const cpBody *body) { return cpTransformPoint(body->transform, cpvzero); }

void cpBodySetPosition(cpBody *body, cpVect position)
{
	/* cpBody.c:374-382 */
	cpBodyActivate(body);
	cpVect p = body->p = cpvadd(cpTransformVect(body->transform, body->cog), position);
	body_set_transform(body, p, body->a);
}

cpVect cpBodyGetCenterOfGravity(const cpBody *body) { return body->cog; }
void cpBodySetCenterOfGravity(cpBody *body, cpVect cog) { cpBodyActivate(body); body->cog = cog; }
cpVect cpBodyGetVelocity(const cpBody *body) { return body->v; }
void cpBodySetVelocity(cpBody *body, cpVect v) { cpBodyActivate(body); body->v = v; }
cpVect cpBodyGetForce(const cpBody *body) { return body->f; }
void cpBodySetForce(cpBody *body, cpVect f) { cpBodyActivate(body); body->f = f; }
cpFloat cpBodyGetAngle(const cpBody *body) { return body->a; }
void cpBodySetAngle(cpBody *body, cpFloat a) { cpBodyActivate(body); body->a = a; body_set_transform(body, body->p, a); }
cpFloat cpBodyGetAngularVelocity(const cpBody *body) { return body->w; }
void cpBodySetAngularVelocity(cpBody *body, cpFloat w) { cpBodyActivate(body); body->w = w; }
cpFloat cpBodyGetTorque(const cpBody *body) { return body->t; }
void cpBodySetTorque(cpBody *body, cpFloat t) { cpBodyActivate(body); body->t = t; }
cpDataPointer cpBodyGetUserData(const cpBody *body) { return body->userData; }
void cpBodySetUserData(cpBody *body, cpDataPointer d) { body->userData = d; }
void cpBodySetVelocityUpdateFunc(cpBody *body, cpBodyVelocityFunc f) { body->velocity_func = f; }
void cpBodySetPositionUpdateFunc(cpBody *body, cpBodyPositionFunc f) { body->position_func = f; }
cpVect cpBodyLocalToWorld(const cpBody *body, const cpVect point) { return cpTransformPoint(body->transform, point); }
cpVect cpBodyWorldToLocal(const cpBody *body, const cpVect point) { return cpTransformPoint(rigid_inverse_(body->transform), point); }

void cpBodyApplyForceAtWorldPoint(cpBody *body, cpVect force, cpVect point)
{
	cpBodyActivate(body);
	body->f = cpvadd(body->f, force);
	cpVect r = cpvsub(point, cpTransformPoint(body->transform, body->cog));
	body->t += cpvcross(r, force);
}

void cpBodyApplyForceAtLocalPoint(cpBody *body, cpVect force, cpVect point)
{
	cpBodyApplyForceAtWorldPoint(body, cpTransformVect(body->transform, force), cpTransformPoint(body->transform, point));
}

/* chipmunk_private.h:193-197 */
static inline void apply_impulse_(cpBody *body, cpVect j, cpVect r)
{
	body->v = cpvadd(body->v, cpvmult(j, body->m_inv));
	body->w += body->i_inv*cpvcross(r, j);
}

static inline void apply_impulses_(cpBody *a, cpBody *b, cpVect r1, cpVect r2, cpVect j)
{
	apply_impulse_(a, cpvneg(j), r1);
	apply_impulse_(b, j, r2);
}

static inline void apply_bias_impulse_(cpBody *body, cpVect j, cpVect r)
{
	body->v_bias = cpvadd(body->v_bias, cpvmult(j, body->m_inv));
	body->w_bias += body->i_inv*cpvcross(r, j);
}

static inline void apply_bias_impulses_(cpBody *a, cpBody *b, cpVect r1, cpVect r2, cpVect j)
{
	apply_bias_impulse_(a, cpvneg(j), r1);
	apply_bias_impulse_(b, j, r2);
}

static inline cpVect relative_velocity_(cpBody *a, cpBody *b, cpVect r1, cpVect r2)
{
	cpVect v1_sum = cpvadd(a->v, cpvmult(cpvperp(r1), a->w));
	cpVect v2_sum = cpvadd(b->v, cpvmult(cpvperp(r2), b->w));
	return cpvsub(v2_sum, v1_sum);
}

static inline cpFloat k_scalar_body_(cpBody *body, cpVect r, cpVect n)
{
	cpFloat rcn = cpvcross(r, n);
	return body->m_inv + body->i_inv*rcn*rcn;
}

static inline cpFloat k_scalar_(cpBody *a, cpBody *b, cpVect r1, cpVect r2, cpVect n)
{
	return k_scalar_body_(a, r1, n) + k_scalar_body_(b, r2, n);
}

/* chipmunk_private.h:228-262 */
static inline cpMat2x2 k_tensor_(cpBody *a, cpBody *b, cpVect r1, cpVect r2)
{
	cpFloat m_sum = a->m_inv + b->m_inv;
	cpFloat k11 = m_sum, k12 = 0.0, k21 = 0.0, k22 = m_sum;
	cpFloat a_i_inv = a->i_inv;
	cpFloat r1xsq = r1.x*r1.x*a_i_inv, r1ysq = r1.y*r1.y*a_i_inv, r1nxy = -r1.x*r1.y*a_i_inv;
	k11 += r1ysq; k12 += r1nxy; k21 += r1nxy; k22 += r1xsq;
	cpFloat b_i_inv = b->i_inv;
	cpFloat r2xsq = r2.x*r2.x*b_i_inv, r2ysq = r2.y*r2.y*b_i_inv, r2nxy = -r2.x*r2.y*b_i_inv;
	k11 += r2ysq; k12 += r2nxy; k21 += r2nxy; k22 += r2xsq;
	cpFloat det = k11*k22 - k12*k21;
	cpFloat det_inv = 1.0/det;
	cpMat2x2 m = { k22*det_inv, -k12*det_inv, -k21*det_inv, k11*det_inv };
	return m;
}

cpVect cpBodyGetVelocityAtWorldPoint(const cpBody *body, cpVect point)
{
	cpVect r = cpvsub(point, cpTransformPoint(body->transform, body->cog));
	return cpvadd(body->v, cpvmult(cpvperp(r), body->w));
}

cpVect cpBodyGetVelocityAtLocalPoint(const cpBody *body, cpVect point)
{
	cpVect r = cpTransformVect(body->transform, cpvsub(point, body->cog));
	return cpvadd(body->v, cpvmult(cpvperp(r), body->w));
}

void cpBodyApplyImpulseAtWorldPoint(cpBody *body, cpVect impulse, cpVect point)
{
	cpBodyActivate(body);
	cpVect r = cpvsub(point, cpTransformPoint(body->transform, body->cog));
	apply_impulse_(body, impulse, r);
}

void cpBodyApplyImpulseAtLocalPoint(cpBody *body, cpVect impulse, cpVect point)
{
	cpBodyApplyImpulseAtWorldPoint(body, cpTransformVect(body->transform, impulse), cpTransformPoint(body->transform, point));
}

cpFloat cpBodyKineticEnergy(const cpBody *body)
{
	cpFloat vsq = cpvdot(body->v, body->v), wsq = body->w*body->w;
	return (vsq ? vsq*body->m : 0.0) + (wsq ? wsq*body->i : 0.0);
}

/* cpBody.c:493-509 */
void cpBodyUpdateVelocity(cpBody *body, cpVect gravity, cpFloat damping, cpFloat dt)
{
	if(body_type(body) == CP_BODY_TYPE_KINEMATIC) return;
	body->v = cpvadd(cpvmult(body->v, damping), cpvmult(cpvadd(gravity, cpvmult(body->f, body->m_inv)), dt));
	body->w = body->w*damping + body->t*body->i_inv*dt;
	body->f = cpvzero;
	body->t = 0.0;
}

/* cpBody.c:511-522 */
void cpBodyUpdatePosition(cpBody *body, cpFloat dt)
{
	cpVect p = body->p = cpvadd(body->p, cpvmult(cpvadd(body->v, body->v_bias), dt));
	cpFloat a = body->a = body->a + (body->w + body->w_bias)*dt;
	body_set_transform(body, p, a);
	body->v_bias = cpvzero;
	body->w_bias = 0.0;
}

void cpBodyEachShape(cpBody *body, cpBodyShapeIteratorFunc func, void *data)
{
	cpShape *s = body->shapeList;
	while(s){ cpShape *next = s->next; func(body, s, data); s = next; }
}

static inline cpConstraint *constraint_next_(cpConstraint *c, cpBody *body) { return (c->a == body ? c->next_a : c->next_b); }

void cpBodyEachConstraint(cpBody *body, cpBodyConstraintIteratorFunc func, void *data)
{
	cpConstraint *c = body->constraintList;
	while(c){ cpConstraint *next = constraint_next_(c, body); func(body, c, data); c = next; }
}

/* Mass from shapes: cpBody.c:206-239 */
static void body_accumulate_mass(cpBody *body)
{
	if(body == NULL || body_type(body) != CP_BODY_TYPE_DYNAMIC) return;
	body->m = body->i = 0.0;
	body->cog = cpvzero;
	cpVect pos = cpBodyGetPosition(body);
	for(cpShape *s = body->shapeList; s; s = s->next){
		cpFloat m = s->mass_m;
		if(m > 0.0){
			cpFloat msum = body->m + m;
			body->i += m*s->mass_i + cpvdistsq(body->cog, s->mass_cog)*(m*body->m)/msum;
			body->cog = cpvlerp(body->cog, s->mass_cog, m/msum);
			body->m = msum;
		}
	}
	body->m_inv = 1.0/body->m;
	body->i_inv = 1.0/body->i;
	cpBodySetPosition(body, pos);
}

/* ========================================================================
 * Shapes: src/cpShape.c, src/cpPolyShape.c
 * ====================================================================== */
static cpShape *shape_new(int kind, cpBody *body, cpFloat m, cpFloat i, cpVect cog, cpFloat area)
{
	/* cpShape.c:28-52 */
	cpShape *s = (cpShape *)calloc(1, sizeof(cpShape));
	s->kind = kind;
	s->body = body;
	s->mass_m = m; s->mass_i = i; s->mass_cog = cog; s->mass_area = area;
	s->filter.group = CP_NO_GROUP;
	s->filter.categories = CP_ALL_CATEGORIES;
	s->filter.mask = CP_ALL_CATEGORIES;
	s->leaf = -1;
	return s;
}

/* cpShape.c:291-296 */
static cpBB circle_cache(cpShape *s, cpTransform t)
{
	cpVect c = s->tc = cpTransformPoint(t, s->c);
	return cpBBNewForCircle(c, s->r);
}

/* cpShape.c:378-405 */
static cpBB segment_cache(cpShape *s, cpTransform t)
{
	s->ta = cpTransformPoint(t, s->sa);
	s->tb = cpTransformPoint(t, s->sb);
	s->tn = cpTransformVect(t, s->sn);
	cpFloat l, r, b, tp;
	if(s->ta.x < s->tb.x){ l = s->ta.x; r = s->tb.x; } else { l = s->tb.x; r = s->ta.x; }
	if(s->ta.y < s->tb.y){ b = s->ta.y; tp = s->tb.y; } else { b = s->tb.y; tp = s->ta.y; }
	cpFloat rad = s->r;
	return cpBBNew(l - rad, b - rad, r + rad, tp + rad);
}

/* cpPolyShape.c:39-64 */
static cpBB poly_cache(cpShape *s, cpTransform t)
{
	int count = s->count;
	cpFloat l = ORC_INF, r = -ORC_INF, b = ORC_INF, tp = -ORC_INF;
	for(int i = 0; i < count; i++){
		cpVect v = cpTransformPoint(t, s->pv[count + i]);
		cpVect n = cpTransformVect(t, s->pn[count + i]);
		s->pv[i] = v;
		s->pn[i] = n;
		l = fmin_(l, v.x); r = fmax_(r, v.x);
		b = fmin_(b, v.y); tp = fmax_(tp, v.y);
	}
	cpFloat rad = s->r;
	return cpBBNew(l - rad, b - rad, r + rad, tp + rad);
}

static cpBB shape_update(cpShape *s, cpTransform t)
{
	switch(s->kind){
		case SHAPE_CIRCLE: return (s->bb = circle_cache(s, t));
		case SHAPE_SEGMENT: return (s->bb = segment_cache(s, t));
		default: return (s->bb = poly_cache(s, t));
	}
}

cpBB cpShapeCacheBB(cpShape *s) { return shape_update(s, s->body->transform); }

cpShape *cpCircleShapeNew(cpBody *body, cpFloat radius, cpVect offset)
{
	/* cpShape.c:313-335 */
	cpShape *s = shape_new(SHAPE_CIRCLE, body, 0.0, cpMomentForCircle(1.0, 0.0, radius, cpvzero), offset, cpAreaForCircle(0.0, radius));
	s->c = offset;
	s->r = radius;
	return s;
}

cpShape *cpSegmentShapeNew(cpBody *body, cpVect a, cpVect b, cpFloat r)
{
	/* cpShape.c:470-502 */
	cpShape *s = shape_new(SHAPE_SEGMENT, body, 0.0, cpMomentForBox(1.0, cpvdist(a, b) + 2.0*r, 2.0*r), cpvlerp(a, b, 0.5), cpAreaForSegment(a, b, r));
	s->sa = a; s->sb = b;
	s->sn = cpvrperp(cpvnormalize(cpvsub(b, a)));
	s->r = r;
	s->a_tangent = cpvzero; s->b_tangent = cpvzero;
	return s;
}

void cpSegmentShapeSetNeighbors(cpShape *s, cpVect prev, cpVect next)
{
	s->a_tangent = cpvsub(prev, s->sa);
	s->b_tangent = cpvsub(next, s->sb);
}

/* cpPolyShape.c:147-165, 175-211 */
cpShape *cpPolyShapeNewRaw(cpBody *body, int count, const cpVect *verts, cpFloat radius)
{
	cpVect centroid = cpCentroidForPoly(count, verts);
	cpShape *s = shape_new(SHAPE_POLY, body, 0.0, cpMomentForPoly(1.0, count, verts, cpvneg(centroid), radius), centroid, cpAreaForPoly(count, verts, radius));
	s->count = count;
	s->pv = (cpVect *)calloc((size_t)(2*count), sizeof(cpVect));
	s->pn = (cpVect *)calloc((size_t)(2*count), sizeof(cpVect));
	for(int i = 0; i < count; i++){
		cpVect a = verts[(i - 1 + count)%count];
		cpVect b = verts[i];
		s->pv[count + i] = b;
		s->pn[count + i] = cpvnormalize(cpvrperp(cpvsub(b, a)));
	}
	s->r = radius;
	return s;
}

/* chipmunk_unsafe.h: shapes changed in place (cpShape.c:553-604,
 * cpPolyShape.c:287-324).  The caches update at the next cpShapeUpdate. */
void cpCircleShapeSetRadius(cpShape *s, cpFloat radius)
{
	ORC_ASSERT(s->kind == SHAPE_CIRCLE, "Shape is not a circle shape.");
	s->r = radius;
	cpFloat mass = s->mass_m;
	s->mass_i = cpMomentForCircle(1.0, 0.0, s->r, cpvzero); s->mass_cog = s->c; s->mass_area = cpAreaForCircle(0.0, s->r);
	if(mass > 0.0) body_accumulate_mass(s->body);
}

void cpCircleShapeSetOffset(cpShape *s, cpVect offset)
{
	ORC_ASSERT(s->kind == SHAPE_CIRCLE, "Shape is not a circle shape.");
	s->c = offset;
	cpFloat mass = s->mass_m;
	s->mass_i = cpMomentForCircle(1.0, 0.0, s->r, cpvzero); s->mass_cog = s->c; s->mass_area = cpAreaForCircle(0.0, s->r);
	if(mass > 0.0) body_accumulate_mass(s->body);
}

/* the normal is cpvperp here, not the constructor's cpvrperp (cpShape.c:586) */
void cpSegmentShapeSetEndpoints(cpShape *s, cpVect a, cpVect b)
{
	ORC_ASSERT(s->kind == SHAPE_SEGMENT, "Shape is not a segment shape.");
	s->sa = a; s->sb = b;
	s->sn = cpvperp(cpvnormalize(cpvsub(b, a)));
	cpFloat mass = s->mass_m;
	s->mass_i = cpMomentForBox(1.0, cpvdist(s->sa, s->sb) + 2.0*s->r, 2.0*s->r);
	s->mass_cog = cpvlerp(s->sa, s->sb, 0.5); s->mass_area = cpAreaForSegment(s->sa, s->sb, s->r);
	if(mass > 0.0) body_accumulate_mass(s->body);
}

void cpSegmentShapeSetRadius(cpShape *s, cpFloat radius)
{
	ORC_ASSERT(s->kind == SHAPE_SEGMENT, "Shape is not a segment shape.");
	s->r = radius;
	cpFloat mass = s->mass_m;
	s->mass_i = cpMomentForBox(1.0, cpvdist(s->sa, s->sb) + 2.0*s->r, 2.0*s->r);
	s->mass_cog = cpvlerp(s->sa, s->sb, 0.5); s->mass_area = cpAreaForSegment(s->sa, s->sb, s->r);
	if(mass > 0.0) body_accumulate_mass(s->body);
}

void cpPolyShapeSetVertsRaw(cpShape *s, int count, cpVect *verts)
{
	ORC_ASSERT(s->kind == SHAPE_POLY, "Shape is not a poly shape.");
	free(s->pv); free(s->pn);
	s->count = count;
	s->pv = (cpVect *)calloc((size_t)(2*count), sizeof(cpVect));
	s->pn = (cpVect *)calloc((size_t)(2*count), sizeof(cpVect));
	for(int i = 0; i < count; i++){
		cpVect a = verts[(i - 1 + count)%count], b = verts[i];
		s->pv[count + i] = b;
		s->pn[count + i] = cpvnormalize(cpvrperp(cpvsub(b, a)));
	}
	cpFloat mass = s->mass_m;
	cpVect centroid = cpCentroidForPoly(count, verts);
	s->mass_i = cpMomentForPoly(1.0, count, verts, cpvneg(centroid), s->r);
	s->mass_cog = centroid; s->mass_area = cpAreaForPoly(count, verts, s->r);
	if(mass > 0.0) body_accumulate_mass(s->body);
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
	ORC_ASSERT(s->kind == SHAPE_POLY, "Shape is not a poly shape.");
	s->r = radius;
}

/* cpShape.c:87-92, 216-220 */
void cpShapeSetBody(cpShape *s, cpBody *body)
{
	ORC_ASSERT(!(s->prev || (s->body && s->body->shapeList == s)), "You cannot change the body on an active shape. You must remove the shape from the space before changing the body.");
	s->body = body;
}

cpBB cpShapeUpdate(cpShape *s, cpTransform transform) { return shape_update(s, transform); }

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

void cpShapeFree(cpShape *s)
{
	if(!s) return;
	free(s->pv); free(s->pn);
	free(s);
}

cpSpace *cpShapeGetSpace(const cpShape *s) { return s->space; }
cpBody *cpShapeGetBody(const cpShape *s) { return s->body; }
cpFloat cpShapeGetMass(cpShape *s) { return s->mass_m; }
void cpShapeSetMass(cpShape *s, cpFloat mass) { cpBodyActivate(s->body); s->mass_m = mass; body_accumulate_mass(s->body); }
cpFloat cpShapeGetDensity(cpShape *s) { return s->mass_m/s->mass_area; }
void cpShapeSetDensity(cpShape *s, cpFloat d) { cpShapeSetMass(s, d*s->mass_area); }
cpFloat cpShapeGetMoment(cpShape *s) { return s->mass_m*s->mass_i; }
cpFloat cpShapeGetArea(cpShape *s) { return s->mass_area; }
cpVect cpShapeGetCenterOfGravity(cpShape *s) { return s->mass_cog; }
cpBB cpShapeGetBB(const cpShape *s) { return s->bb; }
cpBool cpShapeGetSensor(const cpShape *s) { return s->sensor; }
void cpShapeSetSensor(cpShape *s, cpBool v) { cpBodyActivate(s->body); s->sensor = v; }
cpFloat cpShapeGetElasticity(const cpShape *s) { return s->e; }
void cpShapeSetElasticity(cpShape *s, cpFloat e) { ORC_ASSERT(e >= 0.0, "Elasticity must be positive."); cpBodyActivate(s->body); s->e = e; }
cpFloat cpShapeGetFriction(const cpShape *s) { return s->u; }
void cpShapeSetFriction(cpShape *s, cpFloat u) { ORC_ASSERT(u >= 0.0, "Friction must be postive."); cpBodyActivate(s->body); s->u = u; }
cpVect cpShapeGetSurfaceVelocity(const cpShape *s) { return s->surfaceV; }
void cpShapeSetSurfaceVelocity(cpShape *s, cpVect v) { cpBodyActivate(s->body); s->surfaceV = v; }
cpDataPointer cpShapeGetUserData(const cpShape *s) { return s->userData; }
void cpShapeSetUserData(cpShape *s, cpDataPointer d) { s->userData = d; }
cpCollisionType cpShapeGetCollisionType(const cpShape *s) { return s->type; }
void cpShapeSetCollisionType(cpShape *s, cpCollisionType t) { cpBodyActivate(s->body); s->type = t; }
cpShapeFilter cpShapeGetFilter(const cpShape *s) { return s->filter; }
void cpShapeSetFilter(cpShape *s, cpShapeFilter f) { cpBodyActivate(s->body); s->filter = f; }
cpVect cpCircleShapeGetOffset(const cpShape *s) { return s->c; }
cpFloat cpCircleShapeGetRadius(const cpShape *s) { return s->r; }
cpVect cpSegmentShapeGetA(const cpShape *s) { return s->sa; }
cpVect cpSegmentShapeGetB(const cpShape *s) { return s->sb; }
cpVect cpSegmentShapeGetNormal(const cpShape *s) { return s->sn; }
cpFloat cpSegmentShapeGetRadius(const cpShape *s) { return s->r; }
int cpPolyShapeGetCount(const cpShape *s) { return s->count; }
cpVect cpPolyShapeGetVert(const cpShape *s, int i) { return s->pv[s->count + i]; }
cpFloat cpPolyShapeGetRadius(const cpShape *s) { return s->r; }

/* ========================================================================
 * Constraints: src/cpConstraint.c, cpPivotJoint.c, cpPinJoint.c,
 * cpSlideJoint.c
 * ====================================================================== */
static cpConstraint *constraint_new(int kind, cpBody *a, cpBody *b)
{
	/* cpConstraint.c:37-57 */
	cpConstraint *c = (cpConstraint *)calloc(1, sizeof(cpConstraint));
	c->kind = kind;
	c->a = a; c->b = b;
	c->maxForce = ORC_INF;
	c->errorBias = pow((cpFloat)(1.0f - 0.1f), 60.0);   /* float literals, cpConstraint.c:50 */
	c->maxBias = ORC_INF;
	c->collideBodies = cpTrue;
	return c;
}

cpConstraint *cpPivotJointNew2(cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB)
{
	cpConstraint *c = constraint_new(JOINT_PIVOT, a, b);
	c->anchorA = anchorA; c->anchorB = anchorB;
	c->jAcc = cpvzero;
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
	cpConstraint *c = constraint_new(JOINT_PIN, a, b);
	c->anchorA = anchorA; c->anchorB = anchorB;
	cpVect p1 = (a ? cpTransformPoint(a->transform, anchorA) : anchorA);
	cpVect p2 = (b ? cpTransformPoint(b->transform, anchorB) : anchorB);
	c->dist = cpvlength(cpvsub(p2, p1));
	c->jnAcc = 0.0;
	return c;
}

cpConstraint *cpSlideJointNew(cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB, cpFloat min, cpFloat max)
{
	cpConstraint *c = constraint_new(JOINT_SLIDE, a, b);
	c->anchorA = anchorA; c->anchorB = anchorB;
	c->min = min; c->max = max;
	c->jnAcc = 0.0;
	return c;
}

/* cpGrooveJoint.c:119-132 */
cpConstraint *cpGrooveJointNew(cpBody *a, cpBody *b, cpVect groove_a, cpVect groove_b, cpVect anchorB)
{
	cpConstraint *c = constraint_new(JOINT_GROOVE, a, b);
	c->grv_a = groove_a; c->grv_b = groove_b;
	c->grv_n = cpvperp(cpvnormalize(cpvsub(groove_b, groove_a)));
	c->anchorB = anchorB;
	c->jAcc = cpvzero;
	return c;
}

/* cpDampedSpring.c:24-27 (default force), 124-140 */
static cpFloat default_spring_force(cpConstraint *c, cpFloat dist) { return (c->restLength - dist)*c->stiffness; }
cpConstraint *cpDampedSpringNew(cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB, cpFloat restLength, cpFloat stiffness, cpFloat damping)
{
	cpConstraint *c = constraint_new(JOINT_DSPRING, a, b);
	c->anchorA = anchorA; c->anchorB = anchorB;
	c->restLength = restLength; c->stiffness = stiffness; c->damping = damping;
	c->springForceFunc = default_spring_force;
	c->jnAcc = 0.0;
	return c;
}

/* cpDampedRotarySpring.c:24-27 (default torque), 100-115 */
static cpFloat default_spring_torque(cpConstraint *c, cpFloat relativeAngle) { return (relativeAngle - c->restAngle)*c->stiffness; }
cpConstraint *cpDampedRotarySpringNew(cpBody *a, cpBody *b, cpFloat restAngle, cpFloat stiffness, cpFloat damping)
{
	cpConstraint *c = constraint_new(JOINT_DRSPRING, a, b);
	c->restAngle = restAngle; c->stiffness = stiffness; c->damping = damping;
	c->springTorqueFunc = default_spring_torque;
	c->jnAcc = 0.0;
	return c;
}

/* cpRotaryLimitJoint.c:108-119 */
cpConstraint *cpRotaryLimitJointNew(cpBody *a, cpBody *b, cpFloat min, cpFloat max)
{
	cpConstraint *c = constraint_new(JOINT_ROTLIMIT, a, b);
	c->min = min; c->max = max;
	c->jnAcc = 0.0;
	return c;
}

/* cpRatchetJoint.c:111-123 */
cpConstraint *cpRatchetJointNew(cpBody *a, cpBody *b, cpFloat phase, cpFloat ratchet)
{
	cpConstraint *c = constraint_new(JOINT_RATCHET, a, b);
	c->angle = 0.0;
	c->phase = phase; c->ratchet = ratchet;
	c->angle = (b ? b->a : 0.0) - (a ? a->a : 0.0);
	return c;
}

/* cpGearJoint.c:91-102 */
cpConstraint *cpGearJointNew(cpBody *a, cpBody *b, cpFloat phase, cpFloat ratio)
{
	cpConstraint *c = constraint_new(JOINT_GEAR, a, b);
	c->phase = phase; c->ratio = ratio; c->ratio_inv = 1.0/ratio;
	c->jnAcc = 0.0;
	return c;
}

/* cpSimpleMotor.c:87-96 */
cpConstraint *cpSimpleMotorNew(cpBody *a, cpBody *b, cpFloat rate)
{
	cpConstraint *c = constraint_new(JOINT_MOTOR, a, b);
	c->rate = rate;
	c->jnAcc = 0.0;
	return c;
}

cpBool cpConstraintIsGrooveJoint(const cpConstraint *c) { return c->kind == JOINT_GROOVE; }
cpBool cpConstraintIsDampedSpring(const cpConstraint *c) { return c->kind == JOINT_DSPRING; }
cpBool cpConstraintIsDampedRotarySpring(const cpConstraint *c) { return c->kind == JOINT_DRSPRING; }
cpBool cpConstraintIsRotaryLimitJoint(const cpConstraint *c) { return c->kind == JOINT_ROTLIMIT; }
cpBool cpConstraintIsRatchetJoint(const cpConstraint *c) { return c->kind == JOINT_RATCHET; }
cpBool cpConstraintIsGearJoint(const cpConstraint *c) { return c->kind == JOINT_GEAR; }
cpBool cpConstraintIsSimpleMotor(const cpConstraint *c) { return c->kind == JOINT_MOTOR; }
cpVect cpGrooveJointGetGrooveA(const cpConstraint *c) { return c->grv_a; }
void cpGrooveJointSetGrooveA(cpConstraint *c, cpVect v) { activate_bodies_(c); c->grv_a = v; c->grv_n = cpvperp(cpvnormalize(cpvsub(c->grv_b, v))); }
cpVect cpGrooveJointGetGrooveB(const cpConstraint *c) { return c->grv_b; }
void cpGrooveJointSetGrooveB(cpConstraint *c, cpVect v) { activate_bodies_(c); c->grv_b = v; c->grv_n = cpvperp(cpvnormalize(cpvsub(v, c->grv_a))); }
cpVect cpGrooveJointGetAnchorB(const cpConstraint *c) { return c->anchorB; }
void cpGrooveJointSetAnchorB(cpConstraint *c, cpVect v) { activate_bodies_(c); c->anchorB = v; }
cpVect cpDampedSpringGetAnchorA(const cpConstraint *c) { return c->anchorA; }
void cpDampedSpringSetAnchorA(cpConstraint *c, cpVect v) { activate_bodies_(c); c->anchorA = v; }
cpVect cpDampedSpringGetAnchorB(const cpConstraint *c) { return c->anchorB; }
void cpDampedSpringSetAnchorB(cpConstraint *c, cpVect v) { activate_bodies_(c); c->anchorB = v; }
cpFloat cpDampedSpringGetRestLength(const cpConstraint *c) { return c->restLength; }
void cpDampedSpringSetRestLength(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->restLength = v; }
cpFloat cpDampedSpringGetStiffness(const cpConstraint *c) { return c->stiffness; }
void cpDampedSpringSetStiffness(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->stiffness = v; }
cpFloat cpDampedSpringGetDamping(const cpConstraint *c) { return c->damping; }
void cpDampedSpringSetDamping(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->damping = v; }
cpDampedSpringForceFunc cpDampedSpringGetSpringForceFunc(const cpConstraint *c) { return c->springForceFunc; }
void cpDampedSpringSetSpringForceFunc(cpConstraint *c, cpDampedSpringForceFunc f) { activate_bodies_(c); c->springForceFunc = f; }
cpFloat cpDampedRotarySpringGetRestAngle(const cpConstraint *c) { return c->restAngle; }
void cpDampedRotarySpringSetRestAngle(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->restAngle = v; }
cpFloat cpDampedRotarySpringGetStiffness(const cpConstraint *c) { return c->stiffness; }
void cpDampedRotarySpringSetStiffness(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->stiffness = v; }
cpFloat cpDampedRotarySpringGetDamping(const cpConstraint *c) { return c->damping; }
void cpDampedRotarySpringSetDamping(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->damping = v; }
cpDampedRotarySpringTorqueFunc cpDampedRotarySpringGetSpringTorqueFunc(const cpConstraint *c) { return c->springTorqueFunc; }
void cpDampedRotarySpringSetSpringTorqueFunc(cpConstraint *c, cpDampedRotarySpringTorqueFunc f) { activate_bodies_(c); c->springTorqueFunc = f; }
cpFloat cpRotaryLimitJointGetMin(const cpConstraint *c) { return c->min; }
void cpRotaryLimitJointSetMin(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->min = v; }
cpFloat cpRotaryLimitJointGetMax(const cpConstraint *c) { return c->max; }
void cpRotaryLimitJointSetMax(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->max = v; }
cpFloat cpRatchetJointGetAngle(const cpConstraint *c) { return c->angle; }
void cpRatchetJointSetAngle(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->angle = v; }
cpFloat cpRatchetJointGetPhase(const cpConstraint *c) { return c->phase; }
void cpRatchetJointSetPhase(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->phase = v; }
cpFloat cpRatchetJointGetRatchet(const cpConstraint *c) { return c->ratchet; }
void cpRatchetJointSetRatchet(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->ratchet = v; }
cpFloat cpGearJointGetPhase(const cpConstraint *c) { return c->phase; }
void cpGearJointSetPhase(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->phase = v; }
cpFloat cpGearJointGetRatio(const cpConstraint *c) { return c->ratio; }
void cpGearJointSetRatio(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->ratio = v; c->ratio_inv = 1.0/v; }
cpFloat cpSimpleMotorGetRate(const cpConstraint *c) { return c->rate; }
void cpSimpleMotorSetRate(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->rate = v; }

void cpConstraintFree(cpConstraint *c) { free(c); }
cpSpace *cpConstraintGetSpace(const cpConstraint *c) { return c->space; }
cpBody *cpConstraintGetBodyA(const cpConstraint *c) { return c->a; }
cpBody *cpConstraintGetBodyB(const cpConstraint *c) { return c->b; }
cpFloat cpConstraintGetMaxForce(const cpConstraint *c) { return c->maxForce; }
void cpConstraintSetMaxForce(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->maxForce = v; }
cpFloat cpConstraintGetErrorBias(const cpConstraint *c) { return c->errorBias; }
void cpConstraintSetErrorBias(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->errorBias = v; }
cpFloat cpConstraintGetMaxBias(const cpConstraint *c) { return c->maxBias; }
void cpConstraintSetMaxBias(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->maxBias = v; }
cpBool cpConstraintGetCollideBodies(const cpConstraint *c) { return c->collideBodies; }
void cpConstraintSetCollideBodies(cpConstraint *c, cpBool v) { activate_bodies_(c); c->collideBodies = v; }
void cpConstraintSetPreSolveFunc(cpConstraint *c, cpConstraintPreSolveFunc f) { c->preSolve = f; }
cpConstraintPreSolveFunc cpConstraintGetPreSolveFunc(const cpConstraint *c) { return c->preSolve; }
cpConstraintPostSolveFunc cpConstraintGetPostSolveFunc(const cpConstraint *c) { return c->postSolve; }
void cpConstraintSetPostSolveFunc(cpConstraint *c, cpConstraintPostSolveFunc f) { c->postSolve = f; }
cpDataPointer cpConstraintGetUserData(const cpConstraint *c) { return c->userData; }
void cpConstraintSetUserData(cpConstraint *c, cpDataPointer d) { c->userData = d; }
cpBool cpConstraintIsPivotJoint(const cpConstraint *c) { return c->kind == JOINT_PIVOT; }
cpBool cpConstraintIsPinJoint(const cpConstraint *c) { return c->kind == JOINT_PIN; }
cpBool cpConstraintIsSlideJoint(const cpConstraint *c) { return c->kind == JOINT_SLIDE; }
cpVect cpPivotJointGetAnchorA(const cpConstraint *c) { return c->anchorA; }
cpVect cpPivotJointGetAnchorB(const cpConstraint *c) { return c->anchorB; }
cpVect cpPinJointGetAnchorA(const cpConstraint *c) { return c->anchorA; }
cpVect cpPinJointGetAnchorB(const cpConstraint *c) { return c->anchorB; }
cpFloat cpPinJointGetDist(const cpConstraint *c) { return c->dist; }
cpVect cpSlideJointGetAnchorA(const cpConstraint *c) { return c->anchorA; }
cpVect cpSlideJointGetAnchorB(const cpConstraint *c) { return c->anchorB; }
/* cpPivotJoint.c:133-155, cpPinJoint.c:109-142, cpSlideJoint.c:127-172:
 * the setters store the value (they also wake the bodies, and no body
 * sleeps here) */
void cpPivotJointSetAnchorA(cpConstraint *c, cpVect v) { activate_bodies_(c); c->anchorA = v; }
void cpPivotJointSetAnchorB(cpConstraint *c, cpVect v) { activate_bodies_(c); c->anchorB = v; }
void cpPinJointSetAnchorA(cpConstraint *c, cpVect v) { activate_bodies_(c); c->anchorA = v; }
void cpPinJointSetAnchorB(cpConstraint *c, cpVect v) { activate_bodies_(c); c->anchorB = v; }
void cpPinJointSetDist(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->dist = v; }
void cpSlideJointSetAnchorA(cpConstraint *c, cpVect v) { activate_bodies_(c); c->anchorA = v; }
void cpSlideJointSetAnchorB(cpConstraint *c, cpVect v) { activate_bodies_(c); c->anchorB = v; }
void cpSlideJointSetMin(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->min = v; }
void cpSlideJointSetMax(cpConstraint *c, cpFloat v) { activate_bodies_(c); c->max = v; }
cpFloat cpSlideJointGetMin(const cpConstraint *c) { return c->min; }
cpFloat cpSlideJointGetMax(const cpConstraint *c) { return c->max; }

cpFloat cpConstraintGetImpulse(cpConstraint *c)
{
	switch(c->kind){
		case JOINT_PIVOT: case JOINT_GROOVE: return cpvlength(c->jAcc);
		case JOINT_DSPRING: case JOINT_DRSPRING: return c->jnAcc;
		default: return fabs_(c->jnAcc);
	}
}

static inline cpFloat bias_coef_(cpFloat errorBias, cpFloat dt) { return 1.0 - pow(errorBias, dt); }

/* cpGrooveJoint.c:24-59, cpDampedSpring.c:29-53, cpDampedRotarySpring.c:29-49,
 * cpRotaryLimitJoint.c:24-46, cpRatchetJoint.c:24-52, cpGearJoint.c:24-35,
 * cpSimpleMotor.c:24-31 (r1 and r2 of the groove and spring are set by the
 * caller only for the spring; the groove computes its own) */
static void joint_prestep_more(cpConstraint *c, cpFloat dt)
{
	cpBody *a = c->a, *b = c->b;
	switch(c->kind){
	case JOINT_GROOVE: {
		cpVect ta = cpTransformPoint(a->transform, c->grv_a);
		cpVect tb = cpTransformPoint(a->transform, c->grv_b);
		cpVect n = cpTransformVect(a->transform, c->grv_n);
		cpFloat d = cpvdot(ta, n);
		c->grv_tn = n;
		c->r2 = cpTransformVect(b->transform, cpvsub(c->anchorB, b->cog));
		cpFloat td = cpvcross(cpvadd(b->p, c->r2), n);
		if(td <= cpvcross(ta, n)){
			c->clamp = 1.0;
			c->r1 = cpvsub(ta, a->p);
		} else if(td >= cpvcross(tb, n)){
			c->clamp = -1.0;
			c->r1 = cpvsub(tb, a->p);
		} else {
			c->clamp = 0.0;
			c->r1 = cpvsub(cpvadd(cpvmult(cpvperp(n), -td), cpvmult(n, d)), a->p);
		}
		c->k = k_tensor_(a, b, c->r1, c->r2);
		cpVect delta = cpvsub(cpvadd(b->p, c->r2), cpvadd(a->p, c->r1));
		c->biasv = vclamp_(cpvmult(delta, -bias_coef_(c->errorBias, dt)/dt), c->maxBias);
		break;
	}
	case JOINT_DSPRING: {
		cpVect delta = cpvsub(cpvadd(b->p, c->r2), cpvadd(a->p, c->r1));
		cpFloat dist = cpvlength(delta);
		c->n = cpvmult(delta, 1.0/(dist ? dist : ORC_INF));
		cpFloat k = k_scalar_(a, b, c->r1, c->r2, c->n);
		c->nMass = 1.0/k;
		c->target_vrn = 0.0;
		c->v_coef = 1.0 - exp(-c->damping*dt*k);
		cpFloat f_spring = c->springForceFunc(c, dist);
		cpFloat j_spring = c->jnAcc = f_spring*dt;
		apply_impulses_(a, b, c->r1, c->r2, cpvmult(c->n, j_spring));
		break;
	}
	case JOINT_DRSPRING: {
		cpFloat moment = a->i_inv + b->i_inv;
		c->iSum = 1.0/moment;
		c->w_coef = 1.0 - exp(-c->damping*dt*moment);
		c->target_wrn = 0.0;
		cpFloat j_spring = c->springTorqueFunc(c, a->a - b->a)*dt;
		c->jnAcc = j_spring;
		a->w -= j_spring*a->i_inv;
		b->w += j_spring*b->i_inv;
		break;
	}
	case JOINT_ROTLIMIT: {
		cpFloat dist = b->a - a->a;
		cpFloat pdist = 0.0;
		if(dist > c->max) pdist = c->max - dist;
		else if(dist < c->min) pdist = c->min - dist;
		c->iSum = 1.0/(a->i_inv + b->i_inv);
		cpFloat maxBias = c->maxBias;
		c->bias = fclamp_(-bias_coef_(c->errorBias, dt)*pdist/dt, -maxBias, maxBias);
		if(!c->bias) c->jnAcc = 0.0;
		break;
	}
	case JOINT_RATCHET: {
		cpFloat angle = c->angle, phase = c->phase, ratchet = c->ratchet;
		cpFloat delta = b->a - a->a;
		cpFloat diff = angle - delta;
		cpFloat pdist = 0.0;
		if(diff*ratchet > 0.0) pdist = diff;
		else c->angle = floor((delta - phase)/ratchet)*ratchet + phase;
		c->iSum = 1.0/(a->i_inv + b->i_inv);
		cpFloat maxBias = c->maxBias;
		c->bias = fclamp_(-bias_coef_(c->errorBias, dt)*pdist/dt, -maxBias, maxBias);
		if(!c->bias) c->jnAcc = 0.0;
		break;
	}
	case JOINT_GEAR: {
		c->iSum = 1.0/(a->i_inv*c->ratio_inv + c->ratio*b->i_inv);
		cpFloat maxBias = c->maxBias;
		c->bias = fclamp_(-bias_coef_(c->errorBias, dt)*(b->a*c->ratio - a->a - c->phase)/dt, -maxBias, maxBias);
		break;
	}
	default: /* JOINT_MOTOR */
		c->iSum = 1.0/(a->i_inv + b->i_inv);
		break;
	}
}

/* cpPivotJoint.c:24-39, cpPinJoint.c:24-46, cpSlideJoint.c:24-56 */
static void joint_prestep(cpConstraint *c, cpFloat dt)
{
	cpBody *a = c->a, *b = c->b;
	c->r1 = cpTransformVect(a->transform, cpvsub(c->anchorA, a->cog));
	c->r2 = cpTransformVect(b->transform, cpvsub(c->anchorB, b->cog));
	if(c->kind == JOINT_PIVOT){
		c->k = k_tensor_(a, b, c->r1, c->r2);
		cpVect delta = cpvsub(cpvadd(b->p, c->r2), cpvadd(a->p, c->r1));
		c->biasv = vclamp_(cpvmult(delta, -bias_coef_(c->errorBias, dt)/dt), c->maxBias);
	} else if(c->kind == JOINT_PIN){
		cpVect delta = cpvsub(cpvadd(b->p, c->r2), cpvadd(a->p, c->r1));
		cpFloat dist = cpvlength(delta);
		c->n = cpvmult(delta, 1.0/(dist ? dist : ORC_INF));
		c->nMass = 1.0/k_scalar_(a, b, c->r1, c->r2, c->n);
		cpFloat maxBias = c->maxBias;
		c->bias = fclamp_(-bias_coef_(c->errorBias, dt)*(dist - c->dist)/dt, -maxBias, maxBias);
	} else if(c->kind == JOINT_SLIDE){
		cpVect delta = cpvsub(cpvadd(b->p, c->r2), cpvadd(a->p, c->r1));
		cpFloat dist = cpvlength(delta);
		cpFloat pdist = 0.0;
		if(dist > c->max){
			pdist = dist - c->max;
			c->n = cpvnormalize(delta);
		} else if(dist < c->min){
			pdist = c->min - dist;
			c->n = cpvneg(cpvnormalize(delta));
		} else {
			c->n = cpvzero;
			c->jnAcc = 0.0;
		}
		c->nMass = 1.0/k_scalar_(a, b, c->r1, c->r2, c->n);
		cpFloat maxBias = c->maxBias;
		c->bias = fclamp_(-bias_coef_(c->errorBias, dt)*pdist/dt, -maxBias, maxBias);
	} else {
		joint_prestep_more(c, dt);
	}
}

static void joint_apply_cached(cpConstraint *c, cpFloat dt_coef)
{
	cpBody *a = c->a, *b = c->b;
	switch(c->kind){
	case JOINT_DSPRING: case JOINT_DRSPRING:
		return;      /* cpDampedSpring.c:55, cpDampedRotarySpring.c:51 */
	case JOINT_ROTLIMIT: case JOINT_RATCHET: case JOINT_MOTOR: {
		cpFloat j = c->jnAcc*dt_coef;
		a->w -= j*a->i_inv;
		b->w += j*b->i_inv;
		return;
	}
	case JOINT_GEAR: {
		cpFloat j = c->jnAcc*dt_coef;
		a->w -= j*a->i_inv*c->ratio_inv;
		b->w += j*b->i_inv;
		return;
	}
	default: break;
	}
	if(c->kind == JOINT_PIVOT || c->kind == JOINT_GROOVE){
		apply_impulses_(c->a, c->b, c->r1, c->r2, cpvmult(c->jAcc, dt_coef));
	} else {
		cpVect j = cpvmult(c->n, c->jnAcc*dt_coef);
		apply_impulses_(c->a, c->b, c->r1, c->r2, j);
	}
}

static void joint_apply(cpConstraint *c, cpFloat dt)
{
	cpBody *a = c->a, *b = c->b;
	if(c->kind == JOINT_PIVOT){
		cpVect r1 = c->r1, r2 = c->r2;
		cpVect vr = relative_velocity_(a, b, r1, r2);
		cpVect j = mat2_mul_(c->k, cpvsub(c->biasv, vr));
		cpVect jOld = c->jAcc;
		c->jAcc = vclamp_(cpvadd(c->jAcc, j), c->maxForce*dt);
		j = cpvsub(c->jAcc, jOld);
		apply_impulses_(a, b, c->r1, c->r2, j);
	} else if(c->kind == JOINT_PIN){
		cpVect n = c->n;
		cpFloat vrn = cpvdot(relative_velocity_(a, b, c->r1, c->r2), n);
		cpFloat jnMax = c->maxForce*dt;
		cpFloat jn = (c->bias - vrn)*c->nMass;
		cpFloat jnOld = c->jnAcc;
		c->jnAcc = fclamp_(jnOld + jn, -jnMax, jnMax);
		jn = c->jnAcc - jnOld;
		apply_impulses_(a, b, c->r1, c->r2, cpvmult(n, jn));
	} else if(c->kind == JOINT_GROOVE){
		/* cpGrooveJoint.c:70-94 */
		cpVect r1 = c->r1, r2 = c->r2;
		cpVect vr = relative_velocity_(a, b, r1, r2);
		cpVect j = mat2_mul_(c->k, cpvsub(c->biasv, vr));
		cpVect jOld = c->jAcc;
		cpVect jn = cpvadd(jOld, j);
		cpVect tn = c->grv_tn;
		cpVect jClamp = (c->clamp*cpvcross(jn, tn) > 0.0) ? jn : cpvproject(jn, tn);
		c->jAcc = vclamp_(jClamp, c->maxForce*dt);
		j = cpvsub(c->jAcc, jOld);
		apply_impulses_(a, b, c->r1, c->r2, j);
	} else if(c->kind == JOINT_DSPRING){
		/* cpDampedSpring.c:57-77 */
		cpVect n = c->n, r1 = c->r1, r2 = c->r2;
		cpFloat vrn = cpvdot(relative_velocity_(a, b, r1, r2), n);
		cpFloat v_damp = (c->target_vrn - vrn)*c->v_coef;
		c->target_vrn = vrn + v_damp;
		cpFloat j_damp = v_damp*c->nMass;
		c->jnAcc += j_damp;
		apply_impulses_(a, b, c->r1, c->r2, cpvmult(c->n, j_damp));
	} else if(c->kind == JOINT_DRSPRING){
		/* cpDampedRotarySpring.c:53-72 */
		cpFloat wrn = a->w - b->w;
		cpFloat w_damp = (c->target_wrn - wrn)*c->w_coef;
		c->target_wrn = wrn + w_damp;
		cpFloat j_damp = w_damp*c->iSum;
		c->jnAcc += j_damp;
		a->w += j_damp*a->i_inv;
		b->w -= j_damp*b->i_inv;
	} else if(c->kind == JOINT_ROTLIMIT || c->kind == JOINT_RATCHET){
		/* cpRotaryLimitJoint.c:59-85, cpRatchetJoint.c:64-87 */
		if(!c->bias) return;
		cpFloat wr = b->w - a->w;
		cpFloat jMax = c->maxForce*dt;
		cpFloat j = -(c->bias + wr)*c->iSum;
		cpFloat jOld = c->jnAcc;
		if(c->kind == JOINT_RATCHET){
			cpFloat ratchet = c->ratchet;
			c->jnAcc = fclamp_((jOld + j)*ratchet, 0.0, jMax*fabs_(ratchet))/ratchet;
		} else if(c->bias < 0.0){
			c->jnAcc = fclamp_(jOld + j, 0.0, jMax);
		} else {
			c->jnAcc = fclamp_(jOld + j, -jMax, 0.0);
		}
		j = c->jnAcc - jOld;
		a->w -= j*a->i_inv;
		b->w += j*b->i_inv;
	} else if(c->kind == JOINT_GEAR){
		/* cpGearJoint.c:48-67 */
		cpFloat wr = b->w*c->ratio - a->w;
		cpFloat jMax = c->maxForce*dt;
		cpFloat j = (c->bias - wr)*c->iSum;
		cpFloat jOld = c->jnAcc;
		c->jnAcc = fclamp_(jOld + j, -jMax, jMax);
		j = c->jnAcc - jOld;
		a->w -= j*a->i_inv*c->ratio_inv;
		b->w += j*b->i_inv;
	} else if(c->kind == JOINT_MOTOR){
		/* cpSimpleMotor.c:43-61 */
		cpFloat wr = b->w - a->w + c->rate;
		cpFloat jMax = c->maxForce*dt;
		cpFloat j = -wr*c->iSum;
		cpFloat jOld = c->jnAcc;
		c->jnAcc = fclamp_(jOld + j, -jMax, jMax);
		j = c->jnAcc - jOld;
		a->w -= j*a->i_inv;
		b->w += j*b->i_inv;
	} else {
		if(cpveql(c->n, cpvzero)) return;
		cpVect n = c->n, r1 = c->r1, r2 = c->r2;
		cpVect vr = relative_velocity_(a, b, r1, r2);
		cpFloat vrn = cpvdot(vr, n);
		cpFloat jn = (c->bias - vrn)*c->nMass;
		cpFloat jnOld = c->jnAcc;
		c->jnAcc = fclamp_(jnOld + jn, -c->maxForce*dt, 0.0);
		jn = c->jnAcc - jnOld;
		apply_impulses_(a, b, c->r1, c->r2, cpvmult(n, jn));
	}
}

/* ========================================================================
 * Narrow phase: src/cpCollision.c, src/cpRobust.c
 * ====================================================================== */
typedef struct CollisionInfo {
	cpShape *a, *b;
	cpCollisionID id;
	cpVect n;
	int count;
	Contact arr[2];
} CollisionInfo;

/* cpRobust.c:5-13 */
static cpBool check_point_greater(const cpVect a, const cpVect b, const cpVect c)
{
	return (b.y - a.y)*(a.x + b.x - 2*c.x) > (b.x - a.x)*(a.y + b.y - 2*c.y);
}

static cpBool check_axis(cpVect v0, cpVect v1, cpVect p, cpVect n)
{
	return cpvdot(p, n) <= fmax_(cpvdot(v0, n), cpvdot(v1, n));
}

static void push_contact(CollisionInfo *info, cpVect p1, cpVect p2, cpHashValue hash)
{
	Contact *con = &info->arr[info->count];
	con->r1 = p1; con->r2 = p2; con->hash = hash;
	info->count++;
}

typedef struct SupportPoint { cpVect p; cpCollisionID index; } SupportPoint;
typedef struct MinkowskiPoint { cpVect a, b, ab; cpCollisionID id; } MinkowskiPoint;

/* cpCollision.c:62-76 */
static int poly_support_index(const cpShape *poly, const cpVect n)
{
	cpFloat max = -ORC_INF;
	int index = 0;
	for(int i = 0; i < poly->count; i++){
		cpFloat d = cpvdot(poly->pv[i], n);
		if(d > max){ max = d; index = i; }
	}
	return index;
}

/* cpCollision.c:86-110 */
static SupportPoint shape_support(const cpShape *s, const cpVect n)
{
	SupportPoint sp;
	switch(s->kind){
		case SHAPE_CIRCLE: sp.p = s->tc; sp.index = 0; break;
		case SHAPE_SEGMENT:
			if(cpvdot(s->ta, n) > cpvdot(s->tb, n)){ sp.p = s->ta; sp.index = 0; }
			else { sp.p = s->tb; sp.index = 1; }
			break;
		default: {
			int i = poly_support_index(s, n);
			sp.p = s->pv[i]; sp.index = (cpCollisionID)i;
		}
	}
	return sp;
}

static MinkowskiPoint minkowski(const SupportPoint a, const SupportPoint b)
{
	MinkowskiPoint m = { a.p, b.p, cpvsub(b.p, a.p), (a.index & 0xFF) << 8 | (b.index & 0xFF) };
	return m;
}

typedef struct SupportCtx { const cpShape *s1, *s2; } SupportCtx;

/* cpCollision.c:138-144 */
static MinkowskiPoint support(const SupportCtx *ctx, const cpVect n)
{
	SupportPoint a = shape_support(ctx->s1, cpvneg(n));
	SupportPoint b = shape_support(ctx->s2, n);
	return minkowski(a, b);
}

typedef struct EdgePoint { cpVect p; cpHashValue hash; } EdgePoint;
typedef struct Edge { EdgePoint a, b; cpFloat r; cpVect n; } Edge;

/* cpCollision.c:163-182 */
static Edge support_edge_poly(const cpShape *poly, const cpVect n)
{
	int count = poly->count;
	int i1 = poly_support_index(poly, n);
	int i0 = (i1 - 1 + count)%count;
	int i2 = (i1 + 1)%count;
	cpHashValue hashid = poly->hashid;
	Edge e;
	if(cpvdot(n, poly->pn[i1]) > cpvdot(n, poly->pn[i2])){
		e.a.p = poly->pv[i0]; e.a.hash = HASH_PAIR(hashid, i0);
		e.b.p = poly->pv[i1]; e.b.hash = HASH_PAIR(hashid, i1);
		e.r = poly->r; e.n = poly->pn[i1];
	} else {
		e.a.p = poly->pv[i1]; e.a.hash = HASH_PAIR(hashid, i1);
		e.b.p = poly->pv[i2]; e.b.hash = HASH_PAIR(hashid, i2);
		e.r = poly->r; e.n = poly->pn[i2];
	}
	return e;
}

/* cpCollision.c:184-195 */
static Edge support_edge_segment(const cpShape *seg, const cpVect n)
{
	cpHashValue hashid = seg->hashid;
	Edge e;
	if(cpvdot(seg->tn, n) > 0.0){
		e.a.p = seg->ta; e.a.hash = HASH_PAIR(hashid, 0);
		e.b.p = seg->tb; e.b.hash = HASH_PAIR(hashid, 1);
		e.r = seg->r; e.n = seg->tn;
	} else {
		e.a.p = seg->tb; e.a.hash = HASH_PAIR(hashid, 1);
		e.b.p = seg->ta; e.b.hash = HASH_PAIR(hashid, 0);
		e.r = seg->r; e.n = cpvneg(seg->tn);
	}
	return e;
}

/* cpCollision.c:199-212 */
static inline cpFloat closest_t(const cpVect a, const cpVect b)
{
	cpVect delta = cpvsub(b, a);
	return -fclamp_(cpvdot(delta, cpvadd(a, b))/(cpvlengthsq(delta) + DBL_MIN), -1.0, 1.0);
}

static inline cpVect lerp_t(const cpVect a, const cpVect b, const cpFloat t)
{
	cpFloat ht = 0.5*t;
	return cpvadd(cpvmult(a, 0.5 - ht), cpvmult(b, 0.5 + ht));
}

typedef struct ClosestPoints { cpVect a, b, n; cpFloat d; cpCollisionID id; } ClosestPoints;

/* cpCollision.c:227-258 */
static ClosestPoints closest_points(const MinkowskiPoint v0, const MinkowskiPoint v1)
{
	cpFloat t = closest_t(v0.ab, v1.ab);
	cpVect p = lerp_t(v0.ab, v1.ab, t);
	cpVect pa = lerp_t(v0.a, v1.a, t);
	cpVect pb = lerp_t(v0.b, v1.b, t);
	cpCollisionID id = (v0.id & 0xFFFF) << 16 | (v1.id & 0xFFFF);
	cpVect delta = cpvsub(v1.ab, v0.ab);
	cpVect n = cpvnormalize(cpvrperp(delta));
	cpFloat d = cpvdot(n, p);
	ClosestPoints pts;
	pts.a = pa; pts.b = pb; pts.id = id;
	if(d <= 0.0 || (-1.0 < t && t < 1.0)){
		pts.n = n; pts.d = d;
	} else {
		cpFloat d2 = cpvlength(p);
		pts.n = cpvmult(p, 1.0/(d2 + DBL_MIN));
		pts.d = d2;
	}
	return pts;
}

static inline cpFloat closest_dist(const cpVect v0, const cpVect v1)
{
	return cpvlengthsq(lerp_t(v0, v1, closest_t(v0, v1)));
}

/* EPA, iterative form of EPARecurse (cpCollision.c:270-343).  Each round
 * adds one point, so the hull never exceeds 3 + 30 vertices. */
#define EPA_MAX 30
static ClosestPoints epa(const SupportCtx *ctx, MinkowskiPoint v0, MinkowskiPoint v1, MinkowskiPoint v2)
{
	MinkowskiPoint bufA[EPA_MAX + 8], bufB[EPA_MAX + 8];
	MinkowskiPoint *hull = bufA, *hull2 = bufB;
	int count = 3;
	hull[0] = v0; hull[1] = v1; hull[2] = v2;
	for(int iteration = 1;; iteration++){
		int mini = 0;
		cpFloat minDist = ORC_INF;
		for(int j = 0, i = count - 1; j < count; i = j, j++){
			cpFloat d = closest_dist(hull[i].ab, hull[j].ab);
			if(d < minDist){ minDist = d; mini = i; }
		}
		MinkowskiPoint e0 = hull[mini];
		MinkowskiPoint e1 = hull[(mini + 1)%count];
		MinkowskiPoint p = support(ctx, cpvperp(cpvsub(e1.ab, e0.ab)));
		cpBool duplicate = (p.id == e0.id || p.id == e1.id);
		if(!duplicate && check_point_greater(e0.ab, e1.ab, p.ab) && iteration < EPA_MAX){
			int count2 = 1;
			hull2[0] = p;
			for(int i = 0; i < count; i++){
				int index = (mini + 1 + i)%count;
				cpVect h0 = hull2[count2 - 1].ab;
				cpVect h1 = hull[index].ab;
				cpVect h2 = (i + 1 < count ? hull[(index + 1)%count] : p).ab;
				if(check_point_greater(h0, h2, h1)){
					hull2[count2] = hull[index];
					count2++;
				}
			}
			MinkowskiPoint *tmp = hull; hull = hull2; hull2 = tmp;
			count = count2;
		} else {
			return closest_points(e0, e1);
		}
	}
}

/* GJK, iterative form of GJKRecurse (cpCollision.c:348-392). */
#define GJK_MAX 30
static ClosestPoints gjk_loop(const SupportCtx *ctx, MinkowskiPoint v0, MinkowskiPoint v1)
{
	for(int iteration = 1;;){
		if(iteration > GJK_MAX) return closest_points(v0, v1);
		if(check_point_greater(v1.ab, v0.ab, cpvzero)){
			MinkowskiPoint t = v0; v0 = v1; v1 = t;
			continue;
		}
		cpFloat t = closest_t(v0.ab, v1.ab);
		cpVect n = (-1.0 < t && t < 1.0 ? cpvperp(cpvsub(v1.ab, v0.ab)) : cpvneg(lerp_t(v0.ab, v1.ab, t)));
		MinkowskiPoint p = support(ctx, n);
		if(check_point_greater(p.ab, v0.ab, cpvzero) && check_point_greater(v1.ab, p.ab, cpvzero)){
			return epa(ctx, v0, p, v1);
		}
		if(check_axis(v0.ab, v1.ab, p.ab, n)){
			return closest_points(v0, v1);
		}
		if(closest_dist(v0.ab, p.ab) < closest_dist(p.ab, v1.ab)){
			v1 = p;
		} else {
			v0 = p;
		}
		iteration++;
	}
}

/* cpCollision.c:395-415 */
static SupportPoint shape_point(const cpShape *s, const int i)
{
	SupportPoint sp;
	switch(s->kind){
		case SHAPE_CIRCLE: sp.p = s->tc; sp.index = 0; break;
		case SHAPE_SEGMENT: sp.p = (i == 0 ? s->ta : s->tb); sp.index = (cpCollisionID)i; break;
		default: {
			int index = (i < s->count ? i : 0);
			sp.p = s->pv[index]; sp.index = (cpCollisionID)index;
		}
	}
	return sp;
}

/* cpCollision.c:416-472 */
static ClosestPoints gjk(const SupportCtx *ctx, cpCollisionID *id)
{
	MinkowskiPoint v0, v1;
	if(*id){
		v0 = minkowski(shape_point(ctx->s1, (*id >> 24) & 0xFF), shape_point(ctx->s2, (*id >> 16) & 0xFF));
		v1 = minkowski(shape_point(ctx->s1, (*id >> 8) & 0xFF), shape_point(ctx->s2, (*id) & 0xFF));
	} else {
		cpVect axis = cpvperp(cpvsub(cpBBCenter(ctx->s1->bb), cpBBCenter(ctx->s2->bb)));
		v0 = support(ctx, axis);
		v1 = support(ctx, cpvneg(axis));
	}
	ClosestPoints points = gjk_loop(ctx, v0, v1);
	*id = points.id;
	return points;
}

/* cpCollision.c:477-518 */
static void contact_points(const Edge e1, const Edge e2, const ClosestPoints points, CollisionInfo *info)
{
	cpFloat mindist = e1.r + e2.r;
	if(points.d <= mindist){
		cpVect n = info->n = points.n;
		cpFloat d_e1_a = cpvcross(e1.a.p, n);
		cpFloat d_e1_b = cpvcross(e1.b.p, n);
		cpFloat d_e2_a = cpvcross(e2.a.p, n);
		cpFloat d_e2_b = cpvcross(e2.b.p, n);
		cpFloat e1_denom = 1.0/(d_e1_b - d_e1_a + DBL_MIN);
		cpFloat e2_denom = 1.0/(d_e2_b - d_e2_a + DBL_MIN);
		{
			cpVect p1 = cpvadd(cpvmult(n,  e1.r), cpvlerp(e1.a.p, e1.b.p, fclamp01_((d_e2_b - d_e1_a)*e1_denom)));
			cpVect p2 = cpvadd(cpvmult(n, -e2.r), cpvlerp(e2.a.p, e2.b.p, fclamp01_((d_e1_a - d_e2_a)*e2_denom)));
			cpFloat dist = cpvdot(cpvsub(p2, p1), n);
			if(dist <= 0.0) push_contact(info, p1, p2, HASH_PAIR(e1.a.hash, e2.b.hash));
		}{
			cpVect p1 = cpvadd(cpvmult(n,  e1.r), cpvlerp(e1.a.p, e1.b.p, fclamp01_((d_e2_a - d_e1_a)*e1_denom)));
			cpVect p2 = cpvadd(cpvmult(n, -e2.r), cpvlerp(e2.a.p, e2.b.p, fclamp01_((d_e1_b - d_e2_a)*e2_denom)));
			cpFloat dist = cpvdot(cpvsub(p2, p1), n);
			if(dist <= 0.0) push_contact(info, p1, p2, HASH_PAIR(e1.b.hash, e2.a.hash));
		}
	}
}

/* cpCollision.c:525-537 */
static void circle_circle(const cpShape *c1, const cpShape *c2, CollisionInfo *info)
{
	cpFloat mindist = c1->r + c2->r;
	cpVect delta = cpvsub(c2->tc, c1->tc);
	cpFloat distsq = cpvlengthsq(delta);
	if(distsq < mindist*mindist){
		cpFloat dist = sqrt(distsq);
		cpVect n = info->n = (dist ? cpvmult(delta, 1.0/dist) : cpv(1.0, 0.0));
		push_contact(info, cpvadd(c1->tc, cpvmult(n, c1->r)), cpvadd(c2->tc, cpvmult(n, -c2->r)), 0);
	}
}

/* cpCollision.c:539-569 */
static void circle_segment(const cpShape *circle, const cpShape *segment, CollisionInfo *info)
{
	cpVect seg_a = segment->ta, seg_b = segment->tb, center = circle->tc;
	cpVect seg_delta = cpvsub(seg_b, seg_a);
	cpFloat closest_t_ = fclamp01_(cpvdot(seg_delta, cpvsub(center, seg_a))/cpvlengthsq(seg_delta));
	cpVect closest = cpvadd(seg_a, cpvmult(seg_delta, closest_t_));
	cpFloat mindist = circle->r + segment->r;
	cpVect delta = cpvsub(closest, center);
	cpFloat distsq = cpvlengthsq(delta);
	if(distsq < mindist*mindist){
		cpFloat dist = sqrt(distsq);
		cpVect n = info->n = (dist ? cpvmult(delta, 1.0/dist) : segment->tn);
		cpVect rot = cpBodyGetRotation(segment->body);
		if((closest_t_ != 0.0 || cpvdot(n, cpvrotate(segment->a_tangent, rot)) >= 0.0) &&
		   (closest_t_ != 1.0 || cpvdot(n, cpvrotate(segment->b_tangent, rot)) >= 0.0)){
			push_contact(info, cpvadd(center, cpvmult(n, circle->r)), cpvadd(closest, cpvmult(n, -segment->r)), 0);
		}
	}
}

/* cpCollision.c:571-604 */
static void segment_segment(const cpShape *seg1, const cpShape *seg2, CollisionInfo *info)
{
	SupportCtx ctx = { seg1, seg2 };
	ClosestPoints points = gjk(&ctx, &info->id);
	cpVect n = points.n;
	cpVect rot1 = cpBodyGetRotation(seg1->body);
	cpVect rot2 = cpBodyGetRotation(seg2->body);
	if(points.d <= (seg1->r + seg2->r) && (
		(!cpveql(points.a, seg1->ta) || cpvdot(n, cpvrotate(seg1->a_tangent, rot1)) <= 0.0) &&
		(!cpveql(points.a, seg1->tb) || cpvdot(n, cpvrotate(seg1->b_tangent, rot1)) <= 0.0) &&
		(!cpveql(points.b, seg2->ta) || cpvdot(n, cpvrotate(seg2->a_tangent, rot2)) >= 0.0) &&
		(!cpveql(points.b, seg2->tb) || cpvdot(n, cpvrotate(seg2->b_tangent, rot2)) >= 0.0))){
		contact_points(support_edge_segment(seg1, n), support_edge_segment(seg2, cpvneg(n)), points, info);
	}
}

/* cpCollision.c:606-627 */
static void poly_poly(const cpShape *poly1, const cpShape *poly2, CollisionInfo *info)
{
	SupportCtx ctx = { poly1, poly2 };
	ClosestPoints points = gjk(&ctx, &info->id);
	if(points.d - poly1->r - poly2->r <= 0.0){
		contact_points(support_edge_poly(poly1, points.n), support_edge_poly(poly2, cpvneg(points.n)), points, info);
	}
}

/* cpCollision.c:629-659 */
static void segment_poly(const cpShape *seg, const cpShape *poly, CollisionInfo *info)
{
	SupportCtx ctx = { seg, poly };
	ClosestPoints points = gjk(&ctx, &info->id);
	cpVect n = points.n;
	cpVect rot = cpBodyGetRotation(seg->body);
	if(points.d - seg->r - poly->r <= 0.0 && (
		(!cpveql(points.a, seg->ta) || cpvdot(n, cpvrotate(seg->a_tangent, rot)) <= 0.0) &&
		(!cpveql(points.a, seg->tb) || cpvdot(n, cpvrotate(seg->b_tangent, rot)) <= 0.0))){
		contact_points(support_edge_segment(seg, n), support_edge_poly(poly, cpvneg(n)), points, info);
	}
}

/* cpCollision.c:661-679 */
static void circle_poly(const cpShape *circle, const cpShape *poly, CollisionInfo *info)
{
	SupportCtx ctx = { circle, poly };
	ClosestPoints points = gjk(&ctx, &info->id);
	if(points.d <= circle->r + poly->r){
		cpVect n = info->n = points.n;
		push_contact(info, cpvadd(points.a, cpvmult(n, circle->r)), cpvadd(points.b, cpvmult(n, -poly->r)), 0);
	}
}

/* cpCollision.c:701-726: order by kind, then dispatch */
static CollisionInfo collide(cpShape *a, cpShape *b, cpCollisionID id)
{
	CollisionInfo info;
	info.a = a; info.b = b; info.id = id; info.n = cpvzero; info.count = 0;
	if(a->kind > b->kind){ info.a = b; info.b = a; }
	int code = info.a->kind + info.b->kind*3;
	switch(code){
		case 0: circle_circle(info.a, info.b, &info); break;
		case 3: circle_segment(info.a, info.b, &info); break;
		case 4: segment_segment(info.a, info.b, &info); break;
		case 6: circle_poly(info.a, info.b, &info); break;
		case 7: segment_poly(info.a, info.b, &info); break;
		case 8: poly_poly(info.a, info.b, &info); break;
		default: ORC_ASSERT(0, "Internal Error: Shape types are not sorted.");
	}
	return info;
}

/* ========================================================================
 * Arbiter cache (src/cpSpaceStep.c:187-325, src/cpArbiter.c:356-498).
 * The reference keys its cache by shape pointers; only membership matters
 * for results, so this map keys by the pair of shape ids.
 * ====================================================================== */
static uint64_t arb_key(const cpShape *a, const cpShape *b)
{
	uint64_t x = (uint64_t)a->hashid, y = (uint64_t)b->hashid;
	if(x > y){ uint64_t t = x; x = y; y = t; }
	return ((x << 32) | y) + 2;   /* never 0 (empty) or 1 (tombstone) */
}

static uint64_t mix64(uint64_t z)
{
	z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
	z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
	return z ^ (z >> 31);
}

static void amap_grow(cpSpace *sp);

static int amap_find(cpSpace *sp, uint64_t key)
{
	ArbMap *m = &sp->amap;
	if(m->cap == 0) return -1;
	unsigned mask = (unsigned)m->cap - 1;
	for(unsigned h = (unsigned)mix64(key) & mask;; h = (h + 1) & mask){
		if(m->keys[h] == 0) return -1;
		if(m->keys[h] == key) return m->slot[h];
	}
}

static void amap_insert(cpSpace *sp, uint64_t key, int slot)
{
	ArbMap *m = &sp->amap;
	if(m->cap == 0 || 2*(m->used + 1) > m->cap) amap_grow(sp);
	unsigned mask = (unsigned)m->cap - 1;
	unsigned h = (unsigned)mix64(key) & mask;
	while(m->keys[h] > 1) h = (h + 1) & mask;
	if(m->keys[h] == 0) m->used++;
	m->keys[h] = key; m->slot[h] = slot;
}

static void amap_remove(cpSpace *sp, uint64_t key)
{
	ArbMap *m = &sp->amap;
	unsigned mask = (unsigned)m->cap - 1;
	for(unsigned h = (unsigned)mix64(key) & mask;; h = (h + 1) & mask){
		if(m->keys[h] == 0) return;
		if(m->keys[h] == key){ m->keys[h] = 1; return; }
	}
}

static void amap_grow(cpSpace *sp)
{
	ArbMap old = sp->amap;
	int live = 0;
	for(int i = 0; i < old.cap; i++) live += (old.keys[i] > 1);
	int cap = 64;
	while(cap < 4*(live + 1)) cap *= 2;
	sp->amap.cap = cap; sp->amap.used = 0;
	sp->amap.keys = (uint64_t *)calloc((size_t)cap, sizeof(uint64_t));
	sp->amap.slot = (int *)calloc((size_t)cap, sizeof(int));
	for(int i = 0; i < old.cap; i++) if(old.keys[i] > 1) amap_insert(sp, old.keys[i], old.slot[i]);
	free(old.keys); free(old.slot);
}

static int arb_alloc(cpSpace *sp)
{
	if(sp->nfree > 0) return sp->freeList[--sp->nfree];
	if(sp->narbs == sp->caparbs){
		sp->caparbs = sp->caparbs ? 2*sp->caparbs : 256;
		sp->arbs = (cpArbiter *)realloc(sp->arbs, sizeof(cpArbiter)*(size_t)sp->caparbs);
	}
	return sp->narbs++;
}

static void arb_free(cpSpace *sp, int slot)
{
	if(sp->nfree == sp->capfree){
		sp->capfree = sp->capfree ? 2*sp->capfree : 256;
		sp->freeList = (int *)realloc(sp->freeList, sizeof(int)*(size_t)sp->capfree);
	}
	sp->freeList[sp->nfree++] = slot;
	sp->arbs[slot].live = 0;
}

/* cpArbiter.c:260-293 */
static void arb_init(cpArbiter *arb, cpShape *a, cpShape *b)
{
	memset(arb, 0, sizeof(*arb));
	arb->a = a; arb->body_a = a->body;
	arb->b = b; arb->body_b = b->body;
	arb->state = ARB_FIRST;
	arb->live = 1;
}

/* cpArbiter.c:356-414 (default collision handler: no swap) */
static cpCollisionHandler *lookup_handler_(cpSpace *sp, cpCollisionType a, cpCollisionType b, cpCollisionHandler *def);
extern cpCollisionHandler orc_handler_do_nothing_;

static void arb_update(cpSpace *sp, cpArbiter *arb, CollisionInfo *info)
{
	cpShape *a = info->a, *b = info->b;
	arb->a = a; arb->body_a = a->body;
	arb->b = b; arb->body_b = b->body;
	for(int i = 0; i < info->count; i++){
		Contact *con = &info->arr[i];
		con->r1 = cpvsub(con->r1, a->body->p);
		con->r2 = cpvsub(con->r2, b->body->p);
		con->jnAcc = con->jtAcc = 0.0;
		for(int j = 0; j < arb->count; j++){
			Contact *old = &arb->contacts[j];
			if(con->hash == old->hash){
				con->jnAcc = old->jnAcc;
				con->jtAcc = old->jtAcc;
			}
		}
	}
	for(int i = 0; i < info->count; i++) arb->contacts[i] = info->arr[i];
	arb->count = info->count;
	arb->n = info->n;
	arb->e = a->e * b->e;
	arb->u = a->u * b->u;
	cpVect surface_vr = cpvsub(b->surfaceV, a->surfaceV);
	arb->surface_vr = cpvsub(surface_vr, cpvmult(info->n, cpvdot(surface_vr, info->n)));
	/* cpArbiter.c:399-410: the handler of the types in info order; swapped
	 * when they are the other way round from the handler's */
	cpCollisionType typeA = a->type, typeB = b->type;
	cpCollisionHandler *defaultHandler = &sp->defaultHandler;
	cpCollisionHandler *handler = arb->handler = lookup_handler_(sp, typeA, typeB, defaultHandler);
	cpBool swapped = arb->swapped = (typeA != handler->typeA && handler->typeA != CP_WILDCARD_COLLISION_TYPE);
	if(handler != defaultHandler || sp->usesWildcards){
		arb->handlerA = lookup_handler_(sp, (swapped ? typeB : typeA), CP_WILDCARD_COLLISION_TYPE, &orc_handler_do_nothing_);
		arb->handlerB = lookup_handler_(sp, (swapped ? typeA : typeB), CP_WILDCARD_COLLISION_TYPE, &orc_handler_do_nothing_);
	}
	if(arb->state == ARB_CACHED) arb->state = ARB_FIRST;
}

/* cpArbiter.c:416-439 */
static void arb_prestep(cpArbiter *arb, cpFloat dt, cpFloat slop, cpFloat bias)
{
	cpBody *a = arb->body_a, *b = arb->body_b;
	cpVect n = arb->n;
	cpVect body_delta = cpvsub(b->p, a->p);
	for(int i = 0; i < arb->count; i++){
		Contact *con = &arb->contacts[i];
		con->nMass = 1.0/k_scalar_(a, b, con->r1, con->r2, n);
		con->tMass = 1.0/k_scalar_(a, b, con->r1, con->r2, cpvperp(n));
		cpFloat dist = cpvdot(cpvadd(cpvsub(con->r2, con->r1), body_delta), n);
		con->bias = -bias*fmin_(0.0, dist + slop)/dt;
		con->jBias = 0.0;
		con->bounce = cpvdot(relative_velocity_(a, b, con->r1, con->r2), n)*arb->e;
	}
}

/* cpArbiter.c:441-455 */
static void arb_apply_cached(cpArbiter *arb, cpFloat dt_coef)
{
	if(arb->state == ARB_FIRST) return;
	cpBody *a = arb->body_a, *b = arb->body_b;
	cpVect n = arb->n;
	for(int i = 0; i < arb->count; i++){
		Contact *con = &arb->contacts[i];
		cpVect j = cpvrotate(n, cpv(con->jnAcc, con->jtAcc));
		apply_impulses_(a, b, con->r1, con->r2, cpvmult(j, dt_coef));
	}
}

/* cpArbiter.c:459-498 */
static void arb_apply(cpArbiter *arb)
{
	cpBody *a = arb->body_a, *b = arb->body_b;
	cpVect n = arb->n;
	cpVect surface_vr = arb->surface_vr;
	cpFloat friction = arb->u;
	for(int i = 0; i < arb->count; i++){
		Contact *con = &arb->contacts[i];
		cpFloat nMass = con->nMass;
		cpVect r1 = con->r1, r2 = con->r2;
		cpVect vb1 = cpvadd(a->v_bias, cpvmult(cpvperp(r1), a->w_bias));
		cpVect vb2 = cpvadd(b->v_bias, cpvmult(cpvperp(r2), b->w_bias));
		cpVect vr = cpvadd(relative_velocity_(a, b, r1, r2), surface_vr);
		cpFloat vbn = cpvdot(cpvsub(vb2, vb1), n);
		cpFloat vrn = cpvdot(vr, n);
		cpFloat vrt = cpvdot(vr, cpvperp(n));
		cpFloat jbn = (con->bias - vbn)*nMass;
		cpFloat jbnOld = con->jBias;
		con->jBias = fmax_(jbnOld + jbn, 0.0);
		cpFloat jn = -(con->bounce + vrn)*nMass;
		cpFloat jnOld = con->jnAcc;
		con->jnAcc = fmax_(jnOld + jn, 0.0);
		cpFloat jtMax = friction*con->jnAcc;
		cpFloat jt = -vrt*con->tMass;
		cpFloat jtOld = con->jtAcc;
		con->jtAcc = fclamp_(jtOld + jt, -jtMax, jtMax);
		apply_bias_impulses_(a, b, r1, r2, cpvmult(n, con->jBias - jbnOld));
		apply_impulses_(a, b, r1, r2, cpvrotate(n, cpv(con->jnAcc - jnOld, con->jtAcc - jtOld)));
	}
}

/* ========================================================================
 * AABB tree with pair cache: src/cpBBTree.c
 * ====================================================================== */
static const int kPrimes[] = {
	/* hash table sizes (src/prime.h:25-55): roughly doubling primes */
	5, 13, 23, 47, 97, 193, 389, 769, 1543, 3079, 6151, 12289, 24593, 49157,
	98317, 196613, 393241, 786433, 1572869, 3145739, 6291469, 12582917,
	25165843, 50331653, 100663319, 201326611, 402653189, 805306457, 1610612741, 0,
};

static unsigned next_prime(unsigned n)
{
	int i = 0;
	while(n > (unsigned)kPrimes[i]){
		i++;
		ORC_ASSERT(kPrimes[i], "hash table too large");
	}
	return (unsigned)kPrimes[i];
}

static void leafset_init(LeafSet *set)
{
	set->size = next_prime(0);
	set->entries = 0;
	set->bins = (int *)malloc(sizeof(int)*set->size);
	for(unsigned i = 0; i < set->size; i++) set->bins[i] = -1;
}

/* cpHashSet.c:87-114 */
static void leafset_resize(cpSpace *sp, LeafSet *set)
{
	unsigned newSize = next_prime(set->size + 1);
	int *bins = (int *)malloc(sizeof(int)*newSize);
	for(unsigned i = 0; i < newSize; i++) bins[i] = -1;
	for(unsigned i = 0; i < set->size; i++){
		int n = set->bins[i];
		while(n >= 0){
			int next = sp->nodes[n].binNext;
			unsigned idx = (unsigned)(sp->nodes[n].obj->hashid % newSize);
			sp->nodes[n].binNext = bins[idx];
			bins[idx] = n;
			n = next;
		}
	}
	free(set->bins);
	set->bins = bins;
	set->size = newSize;
}

static int node_alloc(cpSpace *sp)
{
	if(sp->freeNode >= 0){
		int n = sp->freeNode;
		sp->freeNode = sp->nodes[n].parent;
		return n;
	}
	if(sp->nnodes == sp->capnodes){
		sp->capnodes = sp->capnodes ? 2*sp->capnodes : 256;
		sp->nodes = (Node *)realloc(sp->nodes, sizeof(Node)*(size_t)sp->capnodes);
	}
	return sp->nnodes++;
}

static void node_recycle(cpSpace *sp, int n)
{
	sp->nodes[n].parent = sp->freeNode;
	sp->freeNode = n;
}

static int pair_alloc(cpSpace *sp)
{
	if(sp->freePair >= 0){
		int p = sp->freePair;
		sp->freePair = sp->pairs[p].a.next;
		return p;
	}
	if(sp->npairs == sp->cappairs){
		sp->cappairs = sp->cappairs ? 2*sp->cappairs : 256;
		sp->pairs = (Pair *)realloc(sp->pairs, sizeof(Pair)*(size_t)sp->cappairs);
	}
	return sp->npairs++;
}

static void pair_recycle(cpSpace *sp, int p)
{
	sp->pairs[p].a.next = sp->freePair;
	sp->freePair = p;
}

#define IS_LEAF(sp, n) ((sp)->nodes[n].obj != NULL)

/* cpBBTree.c:82-98: fattened box of a dynamic leaf */
static cpBB leaf_bb(const Tree *tree, const cpShape *s)
{
	cpBB bb = s->bb;
	if(tree->isDynamic){
		/* float literals in the reference: the margin factors are (double)0.1f */
		cpFloat coef = (cpFloat)0.1f;
		cpFloat x = (bb.r - bb.l)*coef;
		cpFloat y = (bb.t - bb.b)*coef;
		cpVect v = cpvmult(s->body->v, (cpFloat)0.1f);
		return cpBBNew(bb.l + fmin_(-x, v.x), bb.b + fmin_(-y, v.y), bb.r + fmax_(x, v.x), bb.t + fmax_(y, v.y));
	}
	return bb;
}

/* cpBBTree.c:150-165 */
static void thread_unlink(cpSpace *sp, Thread thread)
{
	int next = thread.next, prev = thread.prev;
	if(next >= 0){
		Pair *np = &sp->pairs[next];
		if(np->a.leaf == thread.leaf) np->a.prev = prev; else np->b.prev = prev;
	}
	if(prev >= 0){
		Pair *pp = &sp->pairs[prev];
		if(pp->a.leaf == thread.leaf) pp->a.next = next; else pp->b.next = next;
	} else {
		sp->nodes[thread.leaf].pairs = next;
	}
}

/* cpBBTree.c:167-186 */
static void pairs_clear(cpSpace *sp, int leaf)
{
	int p = sp->nodes[leaf].pairs;
	sp->nodes[leaf].pairs = -1;
	while(p >= 0){
		Pair *pr = &sp->pairs[p];
		int next;
		if(pr->a.leaf == leaf){
			next = pr->a.next;
			thread_unlink(sp, pr->b);
		} else {
			next = pr->b.next;
			thread_unlink(sp, pr->a);
		}
		pair_recycle(sp, p);
		p = next;
	}
}

/* cpBBTree.c:188-205 */
static void pair_insert(cpSpace *sp, int a, int b)
{
	int nextA = sp->nodes[a].pairs, nextB = sp->nodes[b].pairs;
	int p = pair_alloc(sp);
	Pair *pr = &sp->pairs[p];
	pr->a.prev = -1; pr->a.leaf = a; pr->a.next = nextA;
	pr->b.prev = -1; pr->b.leaf = b; pr->b.next = nextB;
	pr->id = 0;
	sp->nodes[a].pairs = p;
	sp->nodes[b].pairs = p;
	if(nextA >= 0){
		Pair *q = &sp->pairs[nextA];
		if(q->a.leaf == a) q->a.prev = p; else q->b.prev = p;
	}
	if(nextB >= 0){
		Pair *q = &sp->pairs[nextB];
		if(q->a.leaf == b) q->a.prev = p; else q->b.prev = p;
	}
}

/* cpBBTree.c:250-267 */
static int node_new(cpSpace *sp, int a, int b)
{
	int n = node_alloc(sp);
	Node *nd = &sp->nodes[n];
	nd->obj = NULL;
	nd->bb = bbmerge_(sp->nodes[a].bb, sp->nodes[b].bb);
	nd->parent = -1;
	nd->A = a; sp->nodes[a].parent = n;
	nd->B = b; sp->nodes[b].parent = n;
	return n;
}

/* cpBBTree.c:281-299 */
static void node_replace_child(cpSpace *sp, int parent, int child, int value)
{
	Node *pn = &sp->nodes[parent];
	if(pn->A == child){
		node_recycle(sp, pn->A);
		pn->A = value; sp->nodes[value].parent = parent;
	} else {
		node_recycle(sp, pn->B);
		pn->B = value; sp->nodes[value].parent = parent;
	}
	for(int n = parent; n >= 0; n = sp->nodes[n].parent){
		sp->nodes[n].bb = bbmerge_(sp->nodes[sp->nodes[n].A].bb, sp->nodes[sp->nodes[n].B].bb);
	}
}

/* cpBBTree.c:325-350 */
static int subtree_insert(cpSpace *sp, int subtree, int leaf)
{
	if(subtree < 0) return leaf;
	if(IS_LEAF(sp, subtree)) return node_new(sp, leaf, subtree);
	Node *st = &sp->nodes[subtree];
	cpBB lbb = sp->nodes[leaf].bb;
	cpFloat cost_a = cpBBArea(sp->nodes[st->B].bb) + bbmergedarea_(sp->nodes[st->A].bb, lbb);
	cpFloat cost_b = cpBBArea(sp->nodes[st->A].bb) + bbmergedarea_(sp->nodes[st->B].bb, lbb);
	if(cost_a == cost_b){
		cost_a = bbproximity_(sp->nodes[st->A].bb, lbb);
		cost_b = bbproximity_(sp->nodes[st->B].bb, lbb);
	}
	if(cost_b < cost_a){
		int nb = subtree_insert(sp, sp->nodes[subtree].B, leaf);
		sp->nodes[subtree].B = nb; sp->nodes[nb].parent = subtree;
	} else {
		int na = subtree_insert(sp, sp->nodes[subtree].A, leaf);
		sp->nodes[subtree].A = na; sp->nodes[na].parent = subtree;
	}
	sp->nodes[subtree].bb = bbmerge_(sp->nodes[subtree].bb, lbb);
	return subtree;
}

/* cpBBTree.c:397-415 */
static int subtree_remove(cpSpace *sp, int subtree, int leaf)
{
	if(leaf == subtree) return -1;
	int parent = sp->nodes[leaf].parent;
	if(parent == subtree){
		int other = (sp->nodes[subtree].A == leaf ? sp->nodes[subtree].B : sp->nodes[subtree].A);
		sp->nodes[other].parent = sp->nodes[subtree].parent;
		node_recycle(sp, subtree);
		return other;
	}
	int other = (sp->nodes[parent].A == leaf ? sp->nodes[parent].B : sp->nodes[parent].A);
	node_replace_child(sp, sp->nodes[parent].parent, parent, other);
	return subtree;
}

/* ---- marking (cpBBTree.c:418-480) ---- */
typedef struct MarkCtx {
	int staticRoot;
	int collide;      /* 1: run cpSpaceCollideShapes, 0: the void query */
} MarkCtx;

/* debug trace of GJK ids (cpx_dump_narrow_ids) */
static int *g_nid = NULL, g_nid_n = 0, g_nid_cap = 0;
static const cpSpace *g_nid_space = NULL;
static cpCollisionID collide_shapes(cpSpace *sp, cpShape *a, cpShape *b, cpCollisionID id);

static void mark_leaf_query(cpSpace *sp, int subtree, int leaf, int left, MarkCtx *ctx)
{
	if(!cpBBIntersects(sp->nodes[leaf].bb, sp->nodes[subtree].bb)) return;
	if(IS_LEAF(sp, subtree)){
		if(left){
			pair_insert(sp, leaf, subtree);
		} else {
			if(sp->nodes[subtree].stamp < sp->nodes[leaf].stamp) pair_insert(sp, subtree, leaf);
			if(ctx->collide) collide_shapes(sp, sp->nodes[leaf].obj, sp->nodes[subtree].obj, 0);
		}
	} else {
		int A = sp->nodes[subtree].A, B = sp->nodes[subtree].B;
		mark_leaf_query(sp, A, leaf, left, ctx);
		mark_leaf_query(sp, B, leaf, left, ctx);
	}
}

static void mark_leaf(cpSpace *sp, int leaf, MarkCtx *ctx)
{
	if(sp->nodes[leaf].stamp == sp->treeStamp){
		if(ctx->staticRoot >= 0) mark_leaf_query(sp, ctx->staticRoot, leaf, 0, ctx);
		for(int n = leaf; sp->nodes[n].parent >= 0; n = sp->nodes[n].parent){
			int parent = sp->nodes[n].parent;
			if(n == sp->nodes[parent].A){
				mark_leaf_query(sp, sp->nodes[parent].B, leaf, 1, ctx);
			} else {
				mark_leaf_query(sp, sp->nodes[parent].A, leaf, 0, ctx);
			}
		}
	} else {
		int p = sp->nodes[leaf].pairs;
		while(p >= 0){
			if(leaf == sp->pairs[p].b.leaf){
				cpCollisionID id = sp->pairs[p].id;
				if(ctx->collide) id = collide_shapes(sp, sp->nodes[sp->pairs[p].a.leaf].obj, sp->nodes[leaf].obj, id);
				sp->pairs[p].id = id;
				p = sp->pairs[p].b.next;
			} else {
				p = sp->pairs[p].a.next;
			}
		}
	}
}

static void mark_subtree(cpSpace *sp, int subtree, MarkCtx *ctx)
{
	if(IS_LEAF(sp, subtree)){
		mark_leaf(sp, subtree, ctx);
	} else {
		mark_subtree(sp, sp->nodes[subtree].A, ctx);
		mark_subtree(sp, sp->nodes[subtree].B, ctx);
	}
}

/* cpBBTree.c:498-517 */
static int leaf_update(cpSpace *sp, Tree *tree, int leaf)
{
	cpShape *s = sp->nodes[leaf].obj;
	cpBB bb = s->bb;
	if(!cpBBContainsBB(sp->nodes[leaf].bb, bb)){
		sp->nodes[leaf].bb = leaf_bb(tree, s);
		int root = subtree_remove(sp, tree->root, leaf);
		tree->root = subtree_insert(sp, root, leaf);
		pairs_clear(sp, leaf);
		sp->nodes[leaf].stamp = sp->treeStamp;
		return 1;
	}
	return 0;
}

/* cpBBTree.c:605-616 with LeafAddPairs (:521-537) */
static void hash_insert_(cpSpace *sp, Tree *tree, cpShape *s);
static void hash_remove_(cpSpace *sp, Tree *tree, cpShape *s);
static void hash_rehash_(cpSpace *sp, Tree *tree);

static void tree_insert(cpSpace *sp, Tree *tree, cpShape *s)
{
	if(sp->useHash){ hash_insert_(sp, tree, s); return; }
	LeafSet *set = &tree->leaves;
	int leaf = node_alloc(sp);
	Node *nd = &sp->nodes[leaf];
	nd->obj = s;
	nd->bb = leaf_bb(tree, s);
	nd->parent = -1;
	nd->stamp = 0;
	nd->pairs = -1;
	unsigned idx = (unsigned)(s->hashid % set->size);
	nd->binNext = set->bins[idx];
	set->bins[idx] = leaf;
	set->entries++;
	if(set->entries >= set->size) leafset_resize(sp, set);
	s->leaf = leaf;

	tree->root = subtree_insert(sp, tree->root, leaf);
	sp->nodes[leaf].stamp = sp->treeStamp;
	if(tree->isDynamic){
		MarkCtx ctx = { sp->statTree.root, 0 };
		mark_leaf(sp, leaf, &ctx);
	} else if(sp->dynTree.root >= 0){
		MarkCtx ctx = { -1, 0 };
		mark_leaf_query(sp, sp->dynTree.root, leaf, 1, &ctx);
	}
	sp->treeStamp++;
}

/* cpBBTree.c:638-654 */
static void tree_reindex_query(cpSpace *sp)
{
	Tree *tree = &sp->dynTree;
	if(tree->root < 0) return;
	LeafSet *set = &tree->leaves;
	for(unsigned i = 0; i < set->size; i++){
		int n = set->bins[i];
		while(n >= 0){
			int next = sp->nodes[n].binNext;
			leaf_update(sp, tree, n);
			n = next;
		}
	}
	MarkCtx ctx = { sp->statTree.root, 1 };
	mark_subtree(sp, tree->root, &ctx);
	sp->treeStamp++;
}

/* ========================================================================
 * Space: src/cpSpace.c, src/cpSpaceStep.c
 * ====================================================================== */
static void push_ptr_(void ***arr, int *n, int *cap, void *p)
{
	if(*n == *cap){
		*cap = *cap ? 2*(*cap) : 64;
		*arr = (void **)realloc(*arr, sizeof(void *)*(size_t)(*cap));
	}
	(*arr)[(*n)++] = p;
}

cpSpace *cpSpaceNew(void)
{
	/* cpSpace.c:119-178 */
	cpSpace *sp = (cpSpace *)calloc(1, sizeof(cpSpace));
	sp->iterations = 10;
	sp->gravity = cpvzero;
	sp->damping = 1.0;
	/* cpSpace.c:136-137 use float literals: slop is (double)0.1f and the
	 * bias base is the float difference 1.0f - 0.1f. */
	sp->collisionSlop = (cpFloat)0.1f;
	sp->collisionBias = pow((cpFloat)(1.0f - 0.1f), 60.0);
	sp->collisionPersistence = 3;
	sp->sleepTimeThreshold = ORC_INF;
	memcpy(&sp->defaultHandler, &orc_handler_do_nothing_, sizeof(cpCollisionHandler));
	sp->freeNode = -1;
	sp->freePair = -1;
	sp->dynTree.root = -1; sp->dynTree.isDynamic = 1; leafset_init(&sp->dynTree.leaves);
	sp->statTree.root = -1; sp->statTree.isDynamic = 0; leafset_init(&sp->statTree.leaves);
	body_init(&sp->staticBody, 0.0, 0.0);
	body_make_static(&sp->staticBody);
	sp->staticBody.space = sp;
	return sp;
}

static void hasty_stop(cpSpace *sp);

/* cpSpace.c:180-205 (cpSpaceDestroy / cpSpaceFree) */
static void activate_wrap_(cpBody *body, void *unused) { (void)unused; cpBodyActivate(body); }

void cpSpaceDestroy(cpSpace *sp)
{
	if(!sp) return;
	cpSpaceEachBody(sp, activate_wrap_, NULL);
	hasty_stop(sp);
	free(sp->dyn); free(sp->stat); free(sp->cons);
	free(sp->nodes); free(sp->pairs);
	free(sp->dynTree.leaves.bins); free(sp->statTree.leaves.bins);
	free(sp->arbs); free(sp->freeList); free(sp->amap.keys); free(sp->amap.slot); free(sp->active);
	free(sp->candPairs);
	sp->dyn = sp->stat = NULL; sp->cons = NULL; sp->nodes = NULL; sp->pairs = NULL;
	sp->dynTree.leaves.bins = sp->statTree.leaves.bins = NULL;
	sp->arbs = NULL; sp->freeList = NULL; sp->amap.keys = NULL; sp->amap.slot = NULL; sp->active = NULL;
	sp->candPairs = NULL;
	free(sp->post); sp->post = NULL; sp->npost = sp->cappost = 0;
	free(sp->sleeping); free(sp->roused); sp->sleeping = sp->roused = NULL;
	HashGrid *grids[2] = { &sp->dynGrid, &sp->statGrid };
	for(int i = 0; i < 2; i++){ free(grids[i]->cells); free(grids[i]->binHandle); free(grids[i]->binNext); memset(grids[i], 0, sizeof(HashGrid)); }
	for(int i = 0; i < sp->nhandlers; i++) free(sp->handlers[i]);
	free(sp->handlers); sp->handlers = NULL; sp->nhandlers = sp->caphandlers = 0;
	sp->nsleeping = sp->capsleeping = sp->nroused = sp->caproused = 0;
}

void cpSpaceFree(cpSpace *sp)
{
	if(!sp) return;
	cpSpaceDestroy(sp);
	free(sp);
}

int cpSpaceGetIterations(const cpSpace *sp) { return sp->iterations; }
void cpSpaceSetIterations(cpSpace *sp, int it) { ORC_ASSERT(it > 0, "Iterations must be positive and non-zero."); sp->iterations = it; }
cpVect cpSpaceGetGravity(const cpSpace *sp) { return sp->gravity; }
/* cpSpace.c:253-263: the sleeping components are woken as the reference
 * wakes them, walking the array that each activation shrinks */
void cpSpaceSetGravity(cpSpace *sp, cpVect g)
{
	sp->gravity = g;
	for(int i = 0; i < sp->nsleeping; i++) cpBodyActivate(sp->sleeping[i]);
}
cpFloat cpSpaceGetDamping(const cpSpace *sp) { return sp->damping; }
void cpSpaceSetDamping(cpSpace *sp, cpFloat d) { sp->damping = d; }
cpFloat cpSpaceGetIdleSpeedThreshold(const cpSpace *sp) { return sp->idleSpeedThreshold; }
void cpSpaceSetIdleSpeedThreshold(cpSpace *sp, cpFloat v) { sp->idleSpeedThreshold = v; }
cpFloat cpSpaceGetSleepTimeThreshold(const cpSpace *sp) { return sp->sleepTimeThreshold; }
void cpSpaceSetSleepTimeThreshold(cpSpace *sp, cpFloat t) { sp->sleepTimeThreshold = t; }
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
cpBool cpSpaceIsLocked(cpSpace *sp) { return sp->locked > 0; }
cpBool cpSpaceContainsShape(cpSpace *sp, cpShape *s) { return s->space == sp; }
cpBool cpSpaceContainsBody(cpSpace *sp, cpBody *b) { return b->space == sp; }
cpBool cpSpaceContainsConstraint(cpSpace *sp, cpConstraint *c) { return c->space == sp; }

cpBody *cpSpaceAddBody(cpSpace *sp, cpBody *body)
{
	/* cpSpace.c:440-451 */
	ORC_ASSERT(!body->space, "You have already added this body to a space.");
	ORC_ASSERT(!sp->locked, "This operation cannot be done safely during a call to cpSpaceStep() or during a query. Put these calls into a post-step callback.");
	if(body_type(body) == CP_BODY_TYPE_STATIC) push_ptr_((void ***)&sp->stat, &sp->nstat, &sp->capstat, body);
	else push_ptr_((void ***)&sp->dyn, &sp->ndyn, &sp->capdyn, body);
	body->space = sp;
	return body;
}

cpShape *cpSpaceAddShape(cpSpace *sp, cpShape *s)
{
	/* cpSpace.c:417-438 */
	ORC_ASSERT(!s->space, "You have already added this shape to a space.");
	cpBody *body = s->body;
	ORC_ASSERT(body->space == sp, "The shape's body must be added to the space before the shape.");
	ORC_ASSERT(!sp->locked, "This operation cannot be done safely during a call to cpSpaceStep() or during a query. Put these calls into a post-step callback.");
	int isStatic = (body_type(body) == CP_BODY_TYPE_STATIC);
	if(!isStatic) cpBodyActivate(body);
	/* cpBody.c:182-194: push on the body's shape list */
	cpShape *next = body->shapeList;
	if(next) next->prev = s;
	s->next = next;
	body->shapeList = s;
	if(s->mass_m > 0.0) body_accumulate_mass(body);
	s->hashid = sp->shapeIDCounter++;
	shape_update(s, body->transform);
	tree_insert(sp, isStatic ? &sp->statTree : &sp->dynTree, s);
	s->space = sp;
	return s;
}

/* cpSpace.c:662-672 with cpBBTreeReindexObject (cpBBTree.c:676-684): the
 * shape's cache is brought to its body's transform; its leaf, when the
 * space holds one, is updated (LeafUpdate) and given its pairs back
 * (LeafAddPairs, cpBBTree.c:521-537), and the stamp advances. */
void cpSpaceReindexShape(cpSpace *sp, cpShape *s)
{
	cpShapeCacheBB(s);
	if(s->space != sp || s->leaf < 0) return;
	/* a sleeping body's shapes are in the static index */
	int isStatic = (body_type(s->body) == CP_BODY_TYPE_STATIC || cpBodyIsSleeping(s->body));
	Tree *tree = isStatic ? &sp->statTree : &sp->dynTree;
	if(sp->useHash){
		/* cpSpaceHashRehashObject (cpSpaceHash.c:276-286): a new handle */
		hash_remove_(sp, tree, s);
		hash_insert_(sp, tree, s);
		return;
	}
	int leaf = s->leaf;
	if(leaf_update(sp, tree, leaf)){
		if(!isStatic){
			MarkCtx ctx = { sp->statTree.root, 0 };
			mark_leaf(sp, leaf, &ctx);
		} else if(sp->dynTree.root >= 0){
			MarkCtx ctx = { -1, 0 };
			mark_leaf_query(sp, sp->dynTree.root, leaf, 1, &ctx);
		}
	}
	sp->treeStamp++;
}

/* cpSpace.c:674-678, in the body's shape-list order */
void cpSpaceReindexShapesForBody(cpSpace *sp, cpBody *body)
{
	for(cpShape *s = body->shapeList; s; s = s->next) cpSpaceReindexShape(sp, s);
}

/* cpSpace.c:654-660: every static shape's cache updated (cpShapeUpdateFunc
 * over the leaf set), then cpBBTreeReindex of the static tree
 * (cpBBTree.c:638-654 with the void query and no static root): each leaf,
 * in bin order, updated; the tree marked; the stamp advanced. */
void cpSpaceReindexStatic(cpSpace *sp)
{
	Tree *tree = &sp->statTree;
	LeafSet *set = &tree->leaves;
	for(unsigned i = 0; i < set->size; i++)
		for(int n = set->bins[i]; n >= 0; n = sp->nodes[n].binNext) cpShapeCacheBB(sp->nodes[n].obj);
	if(sp->useHash){ hash_rehash_(sp, tree); return; }
	if(tree->root < 0) return;
	for(unsigned i = 0; i < set->size; i++){
		int n = set->bins[i];
		while(n >= 0){
			int next = sp->nodes[n].binNext;
			leaf_update(sp, tree, n);
			n = next;
		}
	}
	MarkCtx ctx = { -1, 0 };
	mark_subtree(sp, tree->root, &ctx);
	sp->treeStamp++;
}

cpConstraint *cpSpaceAddConstraint(cpSpace *sp, cpConstraint *c)
{
	/* cpSpace.c:453-474 */
	ORC_ASSERT(!c->space, "You have already added this constraint to a space.");
	ORC_ASSERT(!sp->locked, "This operation cannot be done safely during a call to cpSpaceStep() or during a query. Put these calls into a post-step callback.");
	cpBody *a = c->a, *b = c->b;
	cpBodyActivate(a);
	cpBodyActivate(b);
	push_ptr_((void ***)&sp->cons, &sp->ncons, &sp->capcons, c);
	c->next_a = a->constraintList; a->constraintList = c;
	c->next_b = b->constraintList; b->constraintList = c;
	c->space = sp;
	return c;
}

/* cpBBTree.c:619-630 (cpBBTreeRemove): the leaf leaves the leaf set
 * (cpHashSet.c:209-233: unlinked from its bin, the others keep their
 * order), the tree and every pair list, and is recycled. */
static void tree_remove(cpSpace *sp, Tree *tree, cpShape *s)
{
	if(sp->useHash){ hash_remove_(sp, tree, s); return; }
	LeafSet *set = &tree->leaves;
	unsigned idx = (unsigned)(s->hashid % set->size);
	int prev = -1, leaf = set->bins[idx];
	while(leaf >= 0 && sp->nodes[leaf].obj != s){ prev = leaf; leaf = sp->nodes[leaf].binNext; }
	ORC_ASSERT(leaf >= 0, "shape missing from its index");
	if(prev >= 0) sp->nodes[prev].binNext = sp->nodes[leaf].binNext;
	else set->bins[idx] = sp->nodes[leaf].binNext;
	set->entries--;
	tree->root = subtree_remove(sp, tree->root, leaf);
	pairs_clear(sp, leaf);
	node_recycle(sp, leaf);
	s->leaf = -1;
}

/* ========================================================================
 * Spatial hash: src/cpSpaceHash.c (cpSpaceUseSpatialHash, cpSpace.c:687-701)
 * ====================================================================== */
/* hash_func (cpSpaceHash.c:223-227): the cell coordinates as cpHashValue */
static unsigned hash_cell_(int x, int y, int n)
{
	return (unsigned)((((cpHashValue)x)*1640531513ul ^ ((cpHashValue)y)*2654435789ul) % (cpHashValue)n);
}

/* floor_int (cpSpaceHash.c:229-235) */
static int floor_int_(cpFloat f)
{
	int i = (int)f;
	return (f < 0.0f && f != i ? i - 1 : i);
}

static void grid_init_(HashGrid *g, cpFloat celldim, int numcells)
{
	free(g->cells); free(g->binHandle); free(g->binNext);
	memset(g, 0, sizeof(*g));
	g->numcells = numcells;
	g->celldim = celldim;
	g->cells = (int *)malloc(sizeof(int)*(size_t)numcells);
	for(int i = 0; i < numcells; i++) g->cells[i] = -1;
	g->freeBin = -1;
	g->stamp = 1;
}

static int grid_bin_(HashGrid *g)
{
	if(g->freeBin >= 0){ int b = g->freeBin; g->freeBin = g->binNext[b]; return b; }
	if(g->nbins == g->capbins){
		g->capbins = g->capbins ? 2*g->capbins : 256;
		g->binHandle = (int *)realloc(g->binHandle, sizeof(int)*(size_t)g->capbins);
		g->binNext = (int *)realloc(g->binNext, sizeof(int)*(size_t)g->capbins);
	}
	return g->nbins++;
}

/* clearTable (cpSpaceHash.c:126-130) */
static void grid_clear_(HashGrid *g)
{
	for(int i = 0; i < g->numcells; i++){
		int b = g->cells[i];
		while(b >= 0){ int next = g->binNext[b]; g->binNext[b] = g->freeBin; g->freeBin = b; b = next; }
		g->cells[i] = -1;
	}
}

static int grid_contains_(const HashGrid *g, int cell, int hand)
{
	for(int b = g->cells[cell]; b >= 0; b = g->binNext[b]) if(g->binHandle[b] == hand) return 1;
	return 0;
}

static void grid_push_(HashGrid *g, int cell, int hand)
{
	int b = grid_bin_(g);
	g->binHandle[b] = hand;
	g->binNext[b] = g->cells[cell];
	g->cells[cell] = b;
}

/* hashHandle (cpSpaceHash.c:237-265) */
static void grid_hash_handle_(HashGrid *g, int hand, cpBB bb)
{
	cpFloat dim = g->celldim;
	int l = floor_int_(bb.l/dim), r = floor_int_(bb.r/dim);
	int b = floor_int_(bb.b/dim), t = floor_int_(bb.t/dim);
	for(int i = l; i <= r; i++){
		for(int j = b; j <= t; j++){
			unsigned idx = hash_cell_(i, j, g->numcells);
			if(grid_contains_(g, (int)idx, hand)) continue;
			grid_push_(g, (int)idx, hand);
		}
	}
}

/* A removed handle's bins leave every cell.  The reference unlinks them
 * when a query next walks the cell (remove_orphaned_handles,
 * cpSpaceHash.c:330-349); the other bins keep their order either way. */
static void grid_unlink_(HashGrid *g, int hand)
{
	for(int i = 0; i < g->numcells; i++){
		int *link = &g->cells[i];
		while(*link >= 0){
			int b = *link;
			if(g->binHandle[b] == hand){ *link = g->binNext[b]; g->binNext[b] = g->freeBin; g->freeBin = b; }
			else link = &g->binNext[b];
		}
	}
}

/* cpSpaceHashInsert (cpSpaceHash.c:269-274): a new handle at the head of
 * its bin in the handle set, then hashed into the cells of the shape's box */
static void hash_insert_(cpSpace *sp, Tree *tree, cpShape *s)
{
	LeafSet *set = &tree->leaves;
	int hand = node_alloc(sp);
	Node *nd = &sp->nodes[hand];
	memset(nd, 0, sizeof(*nd));
	nd->obj = s;
	nd->parent = -1; nd->A = nd->B = -1; nd->pairs = -1;
	nd->stamp = 0;
	unsigned idx = (unsigned)(s->hashid % set->size);
	nd->binNext = set->bins[idx];
	set->bins[idx] = hand;
	set->entries++;
	if(set->entries >= set->size) leafset_resize(sp, set);
	s->leaf = hand;
	grid_hash_handle_(tree->isDynamic ? &sp->dynGrid : &sp->statGrid, hand, s->bb);
}

/* cpSpaceHashRemove (cpSpaceHash.c:300-309) */
static void hash_remove_(cpSpace *sp, Tree *tree, cpShape *s)
{
	LeafSet *set = &tree->leaves;
	unsigned idx = (unsigned)(s->hashid % set->size);
	int prev = -1, hand = set->bins[idx];
	while(hand >= 0 && sp->nodes[hand].obj != s){ prev = hand; hand = sp->nodes[hand].binNext; }
	ORC_ASSERT(hand >= 0, "shape missing from its index");
	if(prev >= 0) sp->nodes[prev].binNext = sp->nodes[hand].binNext;
	else set->bins[idx] = sp->nodes[hand].binNext;
	set->entries--;
	grid_unlink_(tree->isDynamic ? &sp->dynGrid : &sp->statGrid, hand);
	node_recycle(sp, hand);
	s->leaf = -1;
}

/* cpSpaceHashRehash (cpSpaceHash.c:282-287): every handle hashed again,
 * in handle-set order */
static void hash_rehash_(cpSpace *sp, Tree *tree)
{
	HashGrid *g = tree->isDynamic ? &sp->dynGrid : &sp->statGrid;
	grid_clear_(g);
	LeafSet *set = &tree->leaves;
	for(unsigned i = 0; i < set->size; i++)
		for(int n = set->bins[i]; n >= 0; n = sp->nodes[n].binNext) grid_hash_handle_(g, n, sp->nodes[n].obj->bb);
}

/* cpSpaceHashReindexQuery (cpSpaceHash.c:432-441) with cpSpaceCollideShapes:
 * each dynamic handle, in handle-set order, meets the handles already in
 * the cells it covers, then joins them (queryRehash_helper, :394-430);
 * then each queries the static hash (cpSpatialIndexCollideStatic). */
static void hash_reindex_query_(cpSpace *sp)
{
	HashGrid *g = &sp->dynGrid, *sg = &sp->statGrid;
	LeafSet *set = &sp->dynTree.leaves;
	grid_clear_(g);
	for(unsigned i = 0; i < set->size; i++){
		for(int hand = set->bins[i]; hand >= 0; hand = sp->nodes[hand].binNext){
			cpShape *obj = sp->nodes[hand].obj;
			cpBB bb = obj->bb;
			cpFloat dim = g->celldim;
			int l = floor_int_(bb.l/dim), r = floor_int_(bb.r/dim);
			int b = floor_int_(bb.b/dim), t = floor_int_(bb.t/dim);
			for(int ci = l; ci <= r; ci++){
				for(int cj = b; cj <= t; cj++){
					int cell = (int)hash_cell_(ci, cj, g->numcells);
					if(grid_contains_(g, cell, hand)) continue;
					/* query_helper (cpSpaceHash.c:353-372) */
					for(int bn = g->cells[cell]; bn >= 0; bn = g->binNext[bn]){
						int other = g->binHandle[bn];
						if(sp->nodes[other].stamp == g->stamp || sp->nodes[other].obj == obj) continue;
						collide_shapes(sp, obj, sp->nodes[other].obj, 0);
						sp->nodes[other].stamp = g->stamp;
					}
					grid_push_(g, cell, hand);
				}
			}
			g->stamp++;
		}
	}
	if(sp->statTree.leaves.entries == 0) return;
	for(unsigned i = 0; i < set->size; i++){
		for(int hand = set->bins[i]; hand >= 0; hand = sp->nodes[hand].binNext){
			/* cpSpaceHashQuery (cpSpaceHash.c:374-392) on the static hash */
			cpShape *obj = sp->nodes[hand].obj;
			cpBB bb = obj->bb;
			cpFloat dim = sg->celldim;
			int l = floor_int_(bb.l/dim), r = floor_int_(bb.r/dim);
			int b = floor_int_(bb.b/dim), t = floor_int_(bb.t/dim);
			for(int ci = l; ci <= r; ci++){
				for(int cj = b; cj <= t; cj++){
					int cell = (int)hash_cell_(ci, cj, sg->numcells);
					for(int bn = sg->cells[cell]; bn >= 0; bn = sg->binNext[bn]){
						int other = sg->binHandle[bn];
						if(sp->nodes[other].stamp == sg->stamp || sp->nodes[other].obj == obj) continue;
						collide_shapes(sp, obj, sp->nodes[other].obj, 0);
						sp->nodes[other].stamp = sg->stamp;
					}
				}
			}
			sg->stamp++;
		}
	}
}

/* cpSpace.c:687-701: both indices become spatial hashes holding the same
 * shapes, the static ones copied first, each in its old index's order */
void cpSpaceUseSpatialHash(cpSpace *sp, cpFloat dim, int count)
{
	int nstat = (int)sp->statTree.leaves.entries, ndyn = (int)sp->dynTree.leaves.entries;
	cpShape **order = (cpShape **)malloc(sizeof(cpShape *)*(size_t)(nstat + ndyn + 1));
	int k = 0;
	Tree *trees[2] = { &sp->statTree, &sp->dynTree };
	for(int t = 0; t < 2; t++){
		LeafSet *set = &trees[t]->leaves;
		for(unsigned i = 0; i < set->size; i++)
			for(int n = set->bins[i]; n >= 0; n = sp->nodes[n].binNext) order[k++] = sp->nodes[n].obj;
	}
	/* a fresh pool: the trees and their pair cache go */
	sp->nnodes = 0; sp->freeNode = -1;
	sp->npairs = 0; sp->freePair = -1;
	free(sp->dynTree.leaves.bins); free(sp->statTree.leaves.bins);
	sp->dynTree.root = -1; leafset_init(&sp->dynTree.leaves);
	sp->statTree.root = -1; leafset_init(&sp->statTree.leaves);
	sp->useHash = 1;
	grid_init_(&sp->statGrid, dim, (int)next_prime((unsigned)count));
	grid_init_(&sp->dynGrid, dim, (int)next_prime((unsigned)count));
	for(int i = 0; i < k; i++) hash_insert_(sp, i < nstat ? &sp->statTree : &sp->dynTree, order[i]);
	free(order);
}

/* cpArrayDeleteObj (cpArray.c:76-88): the last element takes the hole. */
static int array_delete_(void **arr, int *n, void *obj)
{
	for(int i = 0; i < *n; i++){
		if(arr[i] == obj){ (*n)--; arr[i] = arr[*n]; arr[*n] = NULL; return i; }
	}
	return -1;
}

/* cpSpace.c:481-521 (cpSpaceFilterArbiters with a shape): every cached
 * arbiter of the shape leaves the contact graph and is dropped.  The
 * reference also deletes it from the last step's arbiter array, whose
 * order then depends on the hash set's pointer hashes; here the array
 * keeps its order (the next step empties it, and nothing reads its order
 * before then). */
static void filter_arbiters_of(cpSpace *sp, cpShape *s)
{
	ArbMap *m = &sp->amap;
	for(int h = 0; h < m->cap; h++){
		if(m->keys[h] <= 1) continue;
		int slot = m->slot[h];
		cpArbiter *arb = &sp->arbs[slot];
		if(arb->a != s && arb->b != s) continue;
		if(arb->state != ARB_CACHED){
			/* the arbiter is invalidated: one of its shapes left */
			arb->state = ARB_INVALID;
			cpCollisionHandler *handler = arb->handler;
			handler->separateFunc(arb, sp, handler->userData);
		}
		m->keys[h] = 1;
		arb_unthread_(sp, slot);
		arb_free(sp, slot);
		int k = 0;
		for(int i = 0; i < sp->nactive; i++) if(sp->active[i] != slot) sp->active[k++] = sp->active[i];
		sp->nactive = k;
	}
}

void cpSpaceRemoveShape(cpSpace *sp, cpShape *s)
{
	/* cpSpace.c:523-545 */
	ORC_ASSERT(s->space == sp, "Cannot remove a shape that was not added to the space.");
	ORC_ASSERT(!sp->locked, "This operation cannot be done safely during a call to cpSpaceStep() or during a query. Put these calls into a post-step callback.");
	cpBody *body = s->body;
	int isStatic = (body_type(body) == CP_BODY_TYPE_STATIC);
	if(isStatic) cpBodyActivateStatic(body, s);
	else cpBodyActivate(body);
	/* cpBodyRemoveShape, cpBody.c:306-327 */
	if(s->prev) s->prev->next = s->next; else body->shapeList = s->next;
	if(s->next) s->next->prev = s->prev;
	s->prev = s->next = NULL;
	if(body_type(body) == CP_BODY_TYPE_DYNAMIC && s->mass_m > 0.0) body_accumulate_mass(body);
	filter_arbiters_of(sp, s);
	tree_remove(sp, isStatic ? &sp->statTree : &sp->dynTree, s);
	s->space = NULL;
	s->hashid = 0;
}

void cpSpaceRemoveBody(cpSpace *sp, cpBody *body)
{
	/* cpSpace.c:547-562 */
	ORC_ASSERT(body != &sp->staticBody, "Cannot remove the designated static body for the space.");
	ORC_ASSERT(body->space == sp, "Cannot remove a body that was not added to the space.");
	ORC_ASSERT(!sp->locked, "This operation cannot be done safely during a call to cpSpaceStep() or during a query. Put these calls into a post-step callback.");
	cpBodyActivate(body);
	if(body_type(body) == CP_BODY_TYPE_STATIC) array_delete_((void **)sp->stat, &sp->nstat, body);
	else array_delete_((void **)sp->dyn, &sp->ndyn, body);
	body->space = NULL;
}

/* cpBody.c:272-287 (filterConstraints) */
static cpConstraint *filter_constraints_(cpConstraint *node, cpBody *body, cpConstraint *filter)
{
	if(node == filter) return constraint_next_(node, body);
	if(node->a == body) node->next_a = filter_constraints_(node->next_a, body, filter);
	else node->next_b = filter_constraints_(node->next_b, body, filter);
	return node;
}

void cpSpaceRemoveConstraint(cpSpace *sp, cpConstraint *c)
{
	/* cpSpace.c:564-577 */
	ORC_ASSERT(c->space == sp, "Cannot remove a constraint that was not added to the space.");
	ORC_ASSERT(!sp->locked, "This operation cannot be done safely during a call to cpSpaceStep() or during a query. Put these calls into a post-step callback.");
	cpBodyActivate(c->a);
	cpBodyActivate(c->b);
	array_delete_((void **)sp->cons, &sp->ncons, c);
	c->a->constraintList = filter_constraints_(c->a->constraintList, c->a, c);
	c->b->constraintList = filter_constraints_(c->b->constraintList, c->b, c);
	c->space = NULL;
}

void cpBodySetType(cpBody *body, cpBodyType type)
{
	/* cpBody.c:157-205 */
	cpBodyType oldType = body_type(body);
	if(oldType == type) return;
	if(body->space) ORC_ASSERT(!body->space->locked, "This operation cannot be done safely during a call to cpSpaceStep() or during a query. Put these calls into a post-step callback.");
	body->idleTime = (type == CP_BODY_TYPE_STATIC ? ORC_INF : 0.0);
	if(type == CP_BODY_TYPE_DYNAMIC){
		body->m = body->i = 0.0;
		body->m_inv = body->i_inv = ORC_INF;
		body_accumulate_mass(body);
	} else {
		body->m = body->i = ORC_INF;
		body->m_inv = body->i_inv = 0.0;
		body->v = cpvzero;
		body->w = 0.0;
	}
	cpSpace *sp = body->space;
	if(!sp) return;
	/* activated with its new type (a no-op unless it turned dynamic) */
	if(oldType != CP_BODY_TYPE_STATIC) cpBodyActivate(body);
	int fromStatic = (oldType == CP_BODY_TYPE_STATIC), toStatic = (type == CP_BODY_TYPE_STATIC);
	if(fromStatic != toStatic){
		if(fromStatic){
			array_delete_((void **)sp->stat, &sp->nstat, body);
			push_ptr_((void ***)&sp->dyn, &sp->ndyn, &sp->capdyn, body);
		} else {
			array_delete_((void **)sp->dyn, &sp->ndyn, body);
			push_ptr_((void ***)&sp->stat, &sp->nstat, &sp->capstat, body);
		}
		for(cpShape *s = body->shapeList; s; s = s->next){
			tree_remove(sp, fromStatic ? &sp->statTree : &sp->dynTree, s);
			tree_insert(sp, toStatic ? &sp->statTree : &sp->dynTree, s);
		}
	}
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

static void each_leaf(cpSpace *sp, LeafSet *set, cpSpaceShapeIteratorFunc func, void *data)
{
	for(unsigned i = 0; i < set->size; i++){
		for(int n = set->bins[i]; n >= 0; n = sp->nodes[n].binNext) func(sp->nodes[n].obj, data);
	}
}

void cpSpaceEachShape(cpSpace *sp, cpSpaceShapeIteratorFunc func, void *data)
{
	sp->locked++;
	each_leaf(sp, &sp->dynTree.leaves, func, data);
	each_leaf(sp, &sp->statTree.leaves, func, data);
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

/* cpShape filter test: chipmunk_private.h:144-155 */
static cpBool filter_reject(cpShapeFilter a, cpShapeFilter b)
{
	return ((a.group != 0 && a.group == b.group) || (a.categories & b.mask) == 0 || (b.categories & a.mask) == 0);
}

static void record_candidate(cpSpace *sp, cpShape *a, cpShape *b)
{
	if(sp->ncand + 2 > sp->capcand){
		sp->capcand = sp->capcand ? 2*sp->capcand : 1024;
		sp->candPairs = (int *)realloc(sp->candPairs, sizeof(int)*(size_t)sp->capcand);
	}
	int x = (int)a->hashid, y = (int)b->hashid;
	sp->candPairs[sp->ncand++] = x < y ? x : y;
	sp->candPairs[sp->ncand++] = x < y ? y : x;
}

/* cpSpaceStep.c:204-232 */
static cpBool query_reject(cpShape *a, cpShape *b)
{
	if(!cpBBIntersects(a->bb, b->bb) || a->body == b->body || filter_reject(a->filter, b->filter)) return cpTrue;
	cpBody *ba = a->body, *bb = b->body;
	for(cpConstraint *c = ba->constraintList; c; c = constraint_next_(c, ba)){
		if(!c->collideBodies && ((c->a == ba && c->b == bb) || (c->a == bb && c->b == ba))) return cpTrue;
	}
	return cpFalse;
}

static void active_push(cpSpace *sp, int slot)
{
	if(sp->nactive == sp->capactive){
		sp->capactive = sp->capactive ? 2*sp->capactive : 256;
		sp->active = (int *)realloc(sp->active, sizeof(int)*(size_t)sp->capactive);
	}
	sp->active[sp->nactive++] = slot;
}

/* cpSpaceStep.c:235-289 (default handlers: begin/preSolve accept) */
/* Debug record of every query-callback call of the last step: shapes, the
 * GJK id passed in and the one returned (cpx_dump_narrow_ids). */
static void record_narrow_id(const cpSpace *sp, const cpShape *a, const cpShape *b, cpCollisionID in, cpCollisionID out)
{
	if(g_nid_space != sp) return;
	if(g_nid_n + 4 > g_nid_cap){
		g_nid_cap = g_nid_cap ? 2*g_nid_cap : 4096;
		g_nid = (int *)realloc(g_nid, sizeof(int)*(size_t)g_nid_cap);
	}
	g_nid[g_nid_n++] = (int)a->hashid; g_nid[g_nid_n++] = (int)b->hashid;
	g_nid[g_nid_n++] = (int)in; g_nid[g_nid_n++] = (int)out;
}

static cpCollisionID collide_shapes_(cpSpace *sp, cpShape *a, cpShape *b, cpCollisionID id);
static cpCollisionID collide_shapes(cpSpace *sp, cpShape *a, cpShape *b, cpCollisionID id)
{
	cpCollisionID out = collide_shapes_(sp, a, b, id);
	record_narrow_id(sp, a, b, id, out);
	return out;
}

/* Records (a, b, id in, id out) of the space's last step, 4 ints each, once
 * cpx_trace_narrow_ids(space) has selected the space (one at a time). */
void cpx_trace_narrow_ids(cpSpace *sp) { g_nid_space = sp; g_nid_n = 0; }
int cpx_dump_narrow_ids(cpSpace *sp, int *out, int max)
{
	int n = (g_nid_space == sp) ? g_nid_n/4 : 0;
	for(int i = 0; i < n && i < max; i++) for(int k = 0; k < 4; k++) out[4*i + k] = g_nid[4*i + k];
	return n;
}

static cpCollisionID collide_shapes_(cpSpace *sp, cpShape *a, cpShape *b, cpCollisionID id)
{
	if(cpBBIntersects(a->bb, b->bb)) record_candidate(sp, a, b);
	if(query_reject(a, b)) return id;
	CollisionInfo info = collide(a, b, id);
	if(info.count == 0) return info.id;
	uint64_t key = arb_key(info.a, info.b);
	int slot = amap_find(sp, key);
	if(slot < 0){
		slot = arb_alloc(sp);
		arb_init(&sp->arbs[slot], info.a, info.b);
		amap_insert(sp, key, slot);
	}
	cpArbiter *arb = &sp->arbs[slot];
	arb_update(sp, arb, &info);
	/* cpSpaceStep.c:259-283: begin on the first step of a collision (false:
	 * ignored until separation), then pre-solve */
	cpCollisionHandler *handler = arb->handler;
	if(arb->state == ARB_FIRST && !handler->beginFunc(arb, sp, handler->userData)) cpArbiterIgnore(arb);
	if(arb->state != ARB_IGNORE && handler->preSolveFunc(arb, sp, handler->userData) && arb->state != ARB_IGNORE &&
	   !(a->sensor || b->sensor) && !(a->body->m == ORC_INF && b->body->m == ORC_INF)){
		active_push(sp, slot);
	} else {
		arb->count = 0;
		if(arb->state != ARB_IGNORE) arb->state = ARB_NORMAL;
	}
	arb->stamp = sp->stamp;
	return info.id;
}

/* ========================================================================
 * The contact graph and sleeping: src/cpSpaceComponent.c, cpArbiter.c:222-247
 * ====================================================================== */
#define ARB_AT_(sp, k) (&(sp)->arbs[(k) - 1])   /* k: slot + 1 */

/* cpArbiterThreadForBody (chipmunk_private.h:178-181) */
static int *thread_prev_(cpArbiter *arb, const cpBody *body) { return (arb->body_a == body) ? &arb->prevA : &arb->prevB; }
static int *thread_next_(cpArbiter *arb, const cpBody *body) { return (arb->body_a == body) ? &arb->nextA : &arb->nextB; }

/* cpBodyPushArbiter (cpSpaceComponent.c:168-181) */
static void body_push_arbiter_(cpSpace *sp, cpBody *body, int slot)
{
	int next = body->arbList;
	*thread_next_(&sp->arbs[slot], body) = next;
	if(next) *thread_prev_(ARB_AT_(sp, next), body) = slot + 1;
	body->arbList = slot + 1;
}

/* unthreadHelper (cpArbiter.c:222-241) */
static void unthread_helper_(cpSpace *sp, int slot, cpBody *body)
{
	cpArbiter *arb = &sp->arbs[slot];
	int prev = *thread_prev_(arb, body), next = *thread_next_(arb, body);
	if(prev) *thread_next_(ARB_AT_(sp, prev), body) = next;
	else if(body->arbList == slot + 1) body->arbList = next;
	if(next) *thread_prev_(ARB_AT_(sp, next), body) = prev;
	*thread_prev_(arb, body) = 0;
	*thread_next_(arb, body) = 0;
}

/* cpArbiterUnthread (cpArbiter.c:243-247) */
static void arb_unthread_(cpSpace *sp, int slot)
{
	unthread_helper_(sp, slot, sp->arbs[slot].body_a);
	unthread_helper_(sp, slot, sp->arbs[slot].body_b);
}

/* cpArbiterNext (chipmunk_private.h:183-186), as slot + 1 */
static int arb_next_(cpSpace *sp, int k, const cpBody *body) { return *thread_next_(ARB_AT_(sp, k), body); }

/* cpArrayDeleteObj (cpArray.c:76-88) on the arbiter list */
static void active_delete_(cpSpace *sp, int slot)
{
	for(int i = 0; i < sp->nactive; i++){
		if(sp->active[i] == slot){ sp->active[i] = sp->active[--sp->nactive]; return; }
	}
}

/* cpSpaceActivateBody (cpSpaceComponent.c:28-79): the body goes back on
 * the dynamic array, its shapes from the static to the dynamic index, the
 * arbiters it owns back into the cache and onto the arbiter list, and the
 * constraints it owns back onto the constraint array.  While the space is
 * locked the body waits on the roused list. */
static void space_activate_body_(cpSpace *sp, cpBody *body)
{
	ORC_ASSERT(body_type(body) == CP_BODY_TYPE_DYNAMIC, "Internal error: Attempting to activate a non-dynamic body.");
	if(sp->locked){
		for(int i = 0; i < sp->nroused; i++) if(sp->roused[i] == body) return;
		push_ptr_((void ***)&sp->roused, &sp->nroused, &sp->caproused, body);
		return;
	}
	push_ptr_((void ***)&sp->dyn, &sp->ndyn, &sp->capdyn, body);
	for(cpShape *s = body->shapeList; s; s = s->next){
		tree_remove(sp, &sp->statTree, s);
		tree_insert(sp, &sp->dynTree, s);
	}
	for(int k = body->arbList; k; k = arb_next_(sp, k, body)){
		cpArbiter *arb = ARB_AT_(sp, k);
		cpBody *bodyA = arb->body_a;
		if(body == bodyA || body_type(bodyA) == CP_BODY_TYPE_STATIC){
			amap_insert(sp, arb_key(arb->a, arb->b), k - 1);
			arb->stamp = sp->stamp;
			active_push(sp, k - 1);
		}
	}
	for(cpConstraint *c = body->constraintList; c; c = constraint_next_(c, body)){
		cpBody *bodyA = c->a;
		if(body == bodyA || body_type(bodyA) == CP_BODY_TYPE_STATIC) push_ptr_((void ***)&sp->cons, &sp->ncons, &sp->capcons, c);
	}
}

/* cpSpaceDeactivateBody (cpSpaceComponent.c:81-112); the arbiters keep
 * their contacts in their slots */
static void space_deactivate_body_(cpSpace *sp, cpBody *body)
{
	ORC_ASSERT(body_type(body) == CP_BODY_TYPE_DYNAMIC, "Internal error: Attempting to deactivate a non-dynamic body.");
	array_delete_((void **)sp->dyn, &sp->ndyn, body);
	for(cpShape *s = body->shapeList; s; s = s->next){
		tree_remove(sp, &sp->dynTree, s);
		tree_insert(sp, &sp->statTree, s);
	}
	for(int k = body->arbList; k; k = arb_next_(sp, k, body)){
		cpArbiter *arb = ARB_AT_(sp, k);
		cpBody *bodyA = arb->body_a;
		if(body == bodyA || body_type(bodyA) == CP_BODY_TYPE_STATIC){
			/* cpSpaceUncacheArbiter (cpSpaceStep.c:223-230) */
			amap_remove(sp, arb_key(arb->a, arb->b));
			active_delete_(sp, k - 1);
		}
	}
	for(cpConstraint *c = body->constraintList; c; c = constraint_next_(c, body)){
		cpBody *bodyA = c->a;
		if(body == bodyA || body_type(bodyA) == CP_BODY_TYPE_STATIC) array_delete_((void **)sp->cons, &sp->ncons, c);
	}
}

/* cpSpaceComponent.c:120-153 */
void cpBodyActivate(cpBody *body)
{
	if(body == NULL || body_type(body) != CP_BODY_TYPE_DYNAMIC) return;
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
	if(!sp) return;
	for(int k = body->arbList; k; k = arb_next_(sp, k, body)){
		cpArbiter *arb = ARB_AT_(sp, k);
		cpBody *other = (arb->body_a == body ? arb->body_b : arb->body_a);
		if(body_type(other) != CP_BODY_TYPE_STATIC) other->idleTime = 0.0;
	}
}

/* cpSpaceComponent.c:155-166 */
void cpBodyActivateStatic(cpBody *body, cpShape *filter)
{
	ORC_ASSERT(body_type(body) == CP_BODY_TYPE_STATIC, "cpBodyActivateStatic() called on a non-static body.");
	cpSpace *sp = body->space;
	if(!sp) return;
	for(int k = body->arbList; k; k = arb_next_(sp, k, body)){
		cpArbiter *arb = ARB_AT_(sp, k);
		if(!filter || filter == arb->a || filter == arb->b) cpBodyActivate(arb->body_a == body ? arb->body_b : arb->body_a);
	}
}

/* FloodFillComponent with ComponentAdd (cpSpaceComponent.c:183-212) */
static void flood_fill_(cpSpace *sp, cpBody *root, cpBody *body)
{
	if(body_type(body) != CP_BODY_TYPE_DYNAMIC || body->sleepRoot != NULL) return;
	body->sleepRoot = root;
	if(body != root){
		body->sleepNext = root->sleepNext;
		root->sleepNext = body;
	}
	for(int k = body->arbList; k; k = arb_next_(sp, k, body)){
		cpArbiter *arb = ARB_AT_(sp, k);
		flood_fill_(sp, root, body == arb->body_a ? arb->body_b : arb->body_a);
	}
	for(cpConstraint *c = body->constraintList; c; c = constraint_next_(c, body)) flood_fill_(sp, root, body == c->a ? c->b : c->a);
}

/* cpSpaceProcessComponents (cpSpaceComponent.c:224-307): idle times, the
 * contact graph rebuilt from the arbiter list, bodies woken by contacts
 * with kinematic or sleeping bodies, and components whose bodies have all
 * idled past the threshold put to sleep. */
static void process_components_(cpSpace *sp, cpFloat dt)
{
	int sleep = (sp->sleepTimeThreshold != ORC_INF);
	if(sleep){
		cpFloat dv = sp->idleSpeedThreshold;
		cpFloat dvsq = (dv ? dv*dv : cpvlengthsq(sp->gravity)*dt*dt);
		for(int i = 0; i < sp->ndyn; i++){
			cpBody *body = sp->dyn[i];
			if(body_type(body) != CP_BODY_TYPE_DYNAMIC) continue;
			cpFloat keThreshold = (dvsq ? body->m*dvsq : 0.0);
			body->idleTime = (cpBodyKineticEnergy(body) > keThreshold ? 0.0 : body->idleTime + dt);
		}
	}
	for(int i = 0, count = sp->nactive; i < count; i++){
		int slot = sp->active[i];
		cpBody *a = sp->arbs[slot].body_a, *b = sp->arbs[slot].body_b;
		if(sleep){
			if(body_type(b) == CP_BODY_TYPE_KINEMATIC || cpBodyIsSleeping(a)) cpBodyActivate(a);
			if(body_type(a) == CP_BODY_TYPE_KINEMATIC || cpBodyIsSleeping(b)) cpBodyActivate(b);
		}
		body_push_arbiter_(sp, a, slot);
		body_push_arbiter_(sp, b, slot);
	}
	if(!sleep) return;
	for(int i = 0; i < sp->ncons; i++){
		cpBody *a = sp->cons[i]->a, *b = sp->cons[i]->b;
		if(body_type(b) == CP_BODY_TYPE_KINEMATIC) cpBodyActivate(a);
		if(body_type(a) == CP_BODY_TYPE_KINEMATIC) cpBodyActivate(b);
	}
	for(int i = 0; i < sp->ndyn;){
		cpBody *body = sp->dyn[i];
		if(body->sleepRoot == NULL){
			flood_fill_(sp, body, body);
			/* ComponentActive (cpSpaceComponent.c:214-222) */
			int active = 0;
			for(cpBody *o = body; o; o = o->sleepNext) if(o->idleTime < sp->sleepTimeThreshold){ active = 1; break; }
			if(!active){
				push_ptr_((void ***)&sp->sleeping, &sp->nsleeping, &sp->capsleeping, body);
				for(cpBody *o = body; o; o = o->sleepNext) space_deactivate_body_(sp, o);
				continue;
			}
		}
		i++;
		body->sleepRoot = NULL;
		body->sleepNext = NULL;
	}
}

/* cpSpaceUnlock (cpSpaceStep.c:68-103) without the post-step callbacks:
 * bodies woken while the space was locked are activated */
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
	ORC_ASSERT(body_type(body) == CP_BODY_TYPE_DYNAMIC, "Non-dynamic bodies cannot be put to sleep.");
	cpSpace *sp = body->space;
	ORC_ASSERT(!sp->locked, "Bodies cannot be put to sleep during a query or a call to cpSpaceStep(). Put these calls into a post-step callback.");
	ORC_ASSERT(sp->sleepTimeThreshold < ORC_INF, "Sleeping is not enabled on the space. You cannot sleep a body without setting a sleep time threshold on the space.");
	ORC_ASSERT(group == NULL || cpBodyIsSleeping(group), "Cannot use a non-sleeping body as a group identifier.");
	if(cpBodyIsSleeping(body)){
		ORC_ASSERT(body->sleepRoot == (group ? group->sleepRoot : NULL), "The body is already sleeping and it's group cannot be reassigned.");
		return;
	}
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
		push_ptr_((void ***)&sp->sleeping, &sp->nsleeping, &sp->capsleeping, body);
	}
	array_delete_((void **)sp->dyn, &sp->ndyn, body);
}

/* cpSpaceStep.c:292-325 */
static void filter_arbiters(cpSpace *sp)
{
	ArbMap *m = &sp->amap;
	for(int h = 0; h < m->cap; h++){
		if(m->keys[h] <= 1) continue;
		int slot = m->slot[h];
		cpArbiter *arb = &sp->arbs[slot];
		cpTimestamp ticks = sp->stamp - arb->stamp;
		cpBody *a = arb->body_a, *b = arb->body_b;
		if((body_type(a) == CP_BODY_TYPE_STATIC || cpBodyIsSleeping(a)) && (body_type(b) == CP_BODY_TYPE_STATIC || cpBodyIsSleeping(b))) continue;
		if(ticks >= 1 && arb->state != ARB_CACHED){
			arb->state = ARB_CACHED;
			cpCollisionHandler *handler = arb->handler;
			handler->separateFunc(arb, sp, handler->userData);
		}
		if(ticks >= sp->collisionPersistence){
			arb->count = 0;
			m->keys[h] = 1;
			arb_free(sp, slot);
		}
	}
}

/* cpSpaceStep.c:335-445 */
/* ========================================================================
 * The threaded solver of src/cpHastySpace.c:387-548, 471-497, 679-682, for
 * the CPU baseline only: with two threads each runs half of the
 * iterations (rounded up) over every arbiter and constraint at the same
 * time, updating the shared bodies without synchronisation, as the
 * reference does.  Its results are not deterministic; nothing checks
 * them.  A persistent worker thread waits on a condition variable between
 * steps (the reference's WorkerThreadLoop / RunWorkers).
 * ====================================================================== */
#define HASTY_THRESHOLD 50

struct Hasty {
	pthread_t thread;
	pthread_mutex_t mutex;
	pthread_cond_t work, done;
	int pending, quit, started;
	cpSpace *sp;
	cpFloat dt;
};

static void hasty_iterations(cpSpace *sp, cpFloat dt, int iters)
{
	for(int it = 0; it < iters; it++){
		for(int i = 0; i < sp->nactive; i++) arb_apply(&sp->arbs[sp->active[i]]);
		for(int i = 0; i < sp->ncons; i++) joint_apply(sp->cons[i], dt);
	}
}

static void *hasty_worker(void *arg)
{
	struct Hasty *h = (struct Hasty *)arg;
	pthread_mutex_lock(&h->mutex);
	for(;;){
		while(!h->pending && !h->quit) pthread_cond_wait(&h->work, &h->mutex);
		if(h->quit) break;
		pthread_mutex_unlock(&h->mutex);
		hasty_iterations(h->sp, h->dt, (h->sp->iterations + 1)/2);
		pthread_mutex_lock(&h->mutex);
		h->pending = 0;
		pthread_cond_signal(&h->done);
	}
	pthread_mutex_unlock(&h->mutex);
	return NULL;
}

static void hasty_solve(cpSpace *sp, cpFloat dt)
{
	struct Hasty *h = sp->hasty;
	pthread_mutex_lock(&h->mutex);
	h->dt = dt;
	h->pending = 1;
	pthread_cond_signal(&h->work);
	pthread_mutex_unlock(&h->mutex);
	hasty_iterations(sp, dt, (sp->iterations + 1)/2);
	pthread_mutex_lock(&h->mutex);
	while(h->pending) pthread_cond_wait(&h->done, &h->mutex);
	pthread_mutex_unlock(&h->mutex);
}

static void hasty_stop(cpSpace *sp)
{
	struct Hasty *h = sp->hasty;
	if(!h) return;
	if(h->started){
		pthread_mutex_lock(&h->mutex);
		h->quit = 1;
		pthread_cond_signal(&h->work);
		pthread_mutex_unlock(&h->mutex);
		pthread_join(h->thread, NULL);
	}
	pthread_mutex_destroy(&h->mutex);
	pthread_cond_destroy(&h->work);
	pthread_cond_destroy(&h->done);
	free(h);
	sp->hasty = NULL;
}

/* Test infrastructure: 2 runs the solver on two threads like cpHastySpace
 * (cpHastySpaceSetThreads caps it at 2), 1 restores the serial solver.
 * Returns the thread count in effect. */
int cpx_space_set_hasty(cpSpace *sp, int threads)
{
	if(!sp) return 0;
	if(threads < 2){ hasty_stop(sp); return 1; }
	if(sp->hasty) return 2;
	struct Hasty *h = (struct Hasty *)calloc(1, sizeof(struct Hasty));
	if(!h) return 1;
	h->sp = sp;
	pthread_mutex_init(&h->mutex, NULL);
	pthread_cond_init(&h->work, NULL);
	pthread_cond_init(&h->done, NULL);
	sp->hasty = h;
	if(pthread_create(&h->thread, NULL, hasty_worker, h) != 0){ hasty_stop(sp); return 1; }
	h->started = 1;
	return 2;
}

void cpSpaceStep(cpSpace *sp, cpFloat dt)
{
	if(dt == 0.0) return;
	sp->stamp++;
	cpFloat prev_dt = sp->curr_dt;
	sp->curr_dt = dt;

	/* cpSpaceStep.c:351-360: the arbiters of awake bodies leave the
	 * contact graph */
	for(int i = 0; i < sp->nactive; i++){
		int slot = sp->active[i];
		cpArbiter *arb = &sp->arbs[slot];
		arb->state = ARB_NORMAL;
		if(!cpBodyIsSleeping(arb->body_a) && !cpBodyIsSleeping(arb->body_b)) arb_unthread_(sp, slot);
	}
	sp->nactive = 0;

	sp->locked++;
	sp->ncand = 0;
	if(g_nid_space == sp) g_nid_n = 0;
	for(int i = 0; i < sp->ndyn; i++){
		cpBody *body = sp->dyn[i];
		body->position_func(body, dt);
	}
	/* shape caches: every dynamic leaf (order is irrelevant) */
	LeafSet *set = &sp->dynTree.leaves;
	for(unsigned i = 0; i < set->size; i++){
		for(int n = set->bins[i]; n >= 0; n = sp->nodes[n].binNext) cpShapeCacheBB(sp->nodes[n].obj);
	}
	if(sp->useHash) hash_reindex_query_(sp);
	else tree_reindex_query(sp);
	space_unlock_(sp);

	process_components_(sp, dt);

	sp->locked++;
	filter_arbiters(sp);

	cpFloat slop = sp->collisionSlop;
	cpFloat biasCoef = 1.0 - pow(sp->collisionBias, dt);
	for(int i = 0; i < sp->nactive; i++) arb_prestep(&sp->arbs[sp->active[i]], dt, slop, biasCoef);
	for(int i = 0; i < sp->ncons; i++){
		cpConstraint *c = sp->cons[i];
		if(c->preSolve) c->preSolve(c, sp);
		joint_prestep(c, dt);
	}

	cpFloat damping = pow(sp->damping, dt);
	cpVect gravity = sp->gravity;
	for(int i = 0; i < sp->ndyn; i++){
		cpBody *body = sp->dyn[i];
		body->velocity_func(body, gravity, damping, dt);
	}

	cpFloat dt_coef = (prev_dt == 0.0 ? 0.0 : dt/prev_dt);
	for(int i = 0; i < sp->nactive; i++) arb_apply_cached(&sp->arbs[sp->active[i]], dt_coef);
	for(int i = 0; i < sp->ncons; i++) joint_apply_cached(sp->cons[i], dt_coef);

	if(sp->hasty && sp->nactive + sp->ncons > HASTY_THRESHOLD) hasty_solve(sp, dt);
	else for(int it = 0; it < sp->iterations; it++){
		for(int i = 0; i < sp->nactive; i++) arb_apply(&sp->arbs[sp->active[i]]);
		for(int i = 0; i < sp->ncons; i++) joint_apply(sp->cons[i], dt);
	}

	for(int i = 0; i < sp->ncons; i++){
		cpConstraint *c = sp->cons[i];
		if(c->postSolve) c->postSolve(c, sp);
	}
	/* cpSpaceStep.c:439-444 */
	for(int i = 0; i < sp->nactive; i++){
		cpArbiter *arb = &sp->arbs[sp->active[i]];
		cpCollisionHandler *handler = arb->handler;
		handler->postSolveFunc(arb, sp, handler->userData);
	}
	space_unlock_(sp);
	run_post_step_(sp);
}

/* ========================================================================
 * Collision handlers: src/cpSpace.c:62-103, 378-413, src/cpArbiter.c:249-356
 * ====================================================================== */
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

/* the default handler of a space that uses wildcards, and the do-nothing
 * handler of one that does not (cpSpace.c:90-103) */
static cpCollisionHandler orc_handler_default_ = {
	CP_WILDCARD_COLLISION_TYPE, CP_WILDCARD_COLLISION_TYPE,
	default_begin_, default_pre_solve_, default_post_solve_, default_separate_, NULL
};
cpCollisionHandler orc_handler_do_nothing_ = {
	CP_WILDCARD_COLLISION_TYPE, CP_WILDCARD_COLLISION_TYPE,
	always_collide_, always_collide_, do_nothing_, do_nothing_, NULL
};

/* cpSpaceLookupHandler (cpArbiter.c:348-354): the handler registered for
 * the unordered pair of types */
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
	cpCollisionHandler *h = lookup_handler_(sp, proto->typeA, proto->typeB, NULL);
	if(h) return h;
	h = (cpCollisionHandler *)malloc(sizeof(cpCollisionHandler));
	memcpy(h, proto, sizeof(cpCollisionHandler));
	push_ptr_((void ***)&sp->handlers, &sp->nhandlers, &sp->caphandlers, h);
	return h;
}

static void use_wildcard_default_(cpSpace *sp)
{
	if(!sp->usesWildcards){
		sp->usesWildcards = 1;
		memcpy(&sp->defaultHandler, &orc_handler_default_, sizeof(cpCollisionHandler));
	}
}

cpCollisionHandler *cpSpaceAddDefaultCollisionHandler(cpSpace *sp)
{
	use_wildcard_default_(sp);
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

/* cpArbiter.c:174-238 */
cpBool cpArbiterIgnore(cpArbiter *arb) { arb->state = ARB_IGNORE; return cpFalse; }
void cpArbiterSetRestitution(cpArbiter *arb, cpFloat e) { arb->e = e; }
void cpArbiterSetFriction(cpArbiter *arb, cpFloat u) { arb->u = u; }
void cpArbiterSetSurfaceVelocity(cpArbiter *arb, cpVect vr) { arb->surface_vr = cpvmult(vr, arb->swapped ? -1.0 : 1.0); }
cpDataPointer cpArbiterGetUserData(const cpArbiter *arb) { return arb->data; }
void cpArbiterSetUserData(cpArbiter *arb, cpDataPointer data) { arb->data = data; }
cpBool cpArbiterIsRemoval(const cpArbiter *arb) { return arb->state == ARB_INVALID; }

/* cpArbiter.c:122-139 */
void cpArbiterSetContactPointSet(cpArbiter *arb, cpContactPointSet *set)
{
	int count = set->count;
	ORC_ASSERT(count == arb->count, "The number of contact points cannot be changed.");
	cpBool swapped = arb->swapped;
	arb->n = (swapped ? cpvneg(set->normal) : set->normal);
	for(int i = 0; i < count; i++){
		cpVect p1 = set->points[i].pointA;
		cpVect p2 = set->points[i].pointB;
		arb->contacts[i].r1 = cpvsub(swapped ? p2 : p1, arb->body_a->p);
		arb->contacts[i].r2 = cpvsub(swapped ? p1 : p2, arb->body_b->p);
	}
}

/* ========================================================================
 * Arbiter queries: src/cpArbiter.c:54-155, cpBody.c:612-626
 * ====================================================================== */
int cpArbiterGetCount(const cpArbiter *arb) { return (arb->state < ARB_CACHED ? arb->count : 0); }
cpFloat cpArbiterGetRestitution(const cpArbiter *arb) { return arb->e; }
cpFloat cpArbiterGetFriction(const cpArbiter *arb) { return arb->u; }
cpVect cpArbiterGetSurfaceVelocity(cpArbiter *arb) { return cpvmult(arb->surface_vr, arb->swapped ? -1.0 : 1.0); }
cpBool cpArbiterIsFirstContact(const cpArbiter *arb) { return arb->state == ARB_FIRST; }
cpVect cpArbiterGetNormal(const cpArbiter *arb) { return cpvmult(arb->n, arb->swapped ? -1.0 : 1.0); }
cpVect cpArbiterGetPointA(const cpArbiter *arb, int i) { return cpvadd(arb->body_a->p, arb->contacts[i].r1); }
cpVect cpArbiterGetPointB(const cpArbiter *arb, int i) { return cpvadd(arb->body_b->p, arb->contacts[i].r2); }

cpFloat cpArbiterGetDepth(const cpArbiter *arb, int i)
{
	const Contact *con = &arb->contacts[i];
	return cpvdot(cpvadd(cpvsub(con->r2, con->r1), cpvsub(arb->body_b->p, arb->body_a->p)), arb->n);
}

cpVect cpArbiterTotalImpulse(const cpArbiter *arb)
{
	cpVect n = arb->n, sum = cpvzero;
	for(int i = 0, count = cpArbiterGetCount(arb); i < count; i++){
		const Contact *con = &arb->contacts[i];
		sum = cpvadd(sum, cpvrotate(n, cpv(con->jnAcc, con->jtAcc)));
	}
	return (arb->swapped ? sum : cpvneg(sum));
}

cpFloat cpArbiterTotalKE(const cpArbiter *arb)
{
	cpFloat eCoef = (1 - arb->e)/(1 + arb->e);
	cpFloat sum = 0.0;
	for(int i = 0, count = cpArbiterGetCount(arb); i < count; i++){
		const Contact *con = &arb->contacts[i];
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
	set.count = cpArbiterGetCount(arb);
	cpBool swapped = arb->swapped;
	cpVect n = arb->n;
	set.normal = (swapped ? cpvneg(n) : n);
	for(int i = 0; i < set.count; i++){
		cpVect p1 = cpvadd(arb->body_a->p, arb->contacts[i].r1);
		cpVect p2 = cpvadd(arb->body_b->p, arb->contacts[i].r2);
		set.points[i].pointA = (swapped ? p2 : p1);
		set.points[i].pointB = (swapped ? p1 : p2);
		set.points[i].distance = cpvdot(cpvsub(p2, p1), n);
	}
	return set;
}

/* cpBody.c:612-626: the body's list in the contact graph; swapped is set
 * relative to the body */
void cpBodyEachArbiter(cpBody *body, cpBodyArbiterIteratorFunc func, void *data)
{
	cpSpace *sp = body->space;
	if(!sp) return;
	for(int k = body->arbList; k;){
		cpArbiter *arb = ARB_AT_(sp, k);
		int next = arb_next_(sp, k, body);
		cpBool swapped = arb->swapped;
		arb->swapped = (body == arb->body_b);
		func(body, arb, data);
		arb->swapped = swapped;
		k = next;
	}
}

/* ========================================================================
 * State export in the shared record layouts (see ref_harness.c)
 * ====================================================================== */
int cpx_dump_bodies(cpSpace *sp, double *out, int max)
{
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

int cpx_set_bodies(cpSpace *sp, const double *in, int count)
{
	for(int i = 0; i < sp->ndyn && i < count; i++){
		cpBody *b = sp->dyn[i];
		const double *o = in + 18*i;
		b->p.x = o[0]; b->p.y = o[1]; b->v.x = o[2]; b->v.y = o[3]; b->a = o[4]; b->w = o[5];
		b->f.x = o[6]; b->f.y = o[7]; b->t = o[8]; b->v_bias.x = o[9]; b->v_bias.y = o[10]; b->w_bias = o[11];
		b->transform.a = o[12]; b->transform.b = o[13]; b->transform.c = o[14]; b->transform.d = o[15];
		b->transform.tx = o[16]; b->transform.ty = o[17];
	}
	return sp->ndyn;
}

int cpx_dump_arbiters(cpSpace *sp, double *out, int max)
{
	for(int i = 0; i < sp->nactive && i < max; i++){
		cpArbiter *arb = &sp->arbs[sp->active[i]];
		double *o = out + 34*i;
		memset(o, 0, 34*sizeof(double));
		o[0] = (double)arb->a->hashid; o[1] = (double)arb->b->hashid; o[2] = arb->count; o[3] = arb->state;
		o[4] = arb->n.x; o[5] = arb->n.y; o[6] = arb->e; o[7] = arb->u; o[8] = arb->surface_vr.x; o[9] = arb->surface_vr.y;
		for(int c = 0; c < arb->count; c++){
			Contact *con = &arb->contacts[c];
			double *q = o + 10 + 12*c;
			q[0] = con->r1.x; q[1] = con->r1.y; q[2] = con->r2.x; q[3] = con->r2.y;
			q[4] = con->nMass; q[5] = con->tMass; q[6] = con->bounce; q[7] = con->jnAcc; q[8] = con->jtAcc;
			q[9] = con->jBias; q[10] = con->bias; q[11] = (double)(con->hash & 0xffffffffffffULL);
		}
	}
	return sp->nactive;
}

int cpx_dump_constraints(cpSpace *sp, double *out, int max)
{
	for(int i = 0; i < sp->ncons && i < max; i++){
		cpConstraint *c = sp->cons[i];
		double *o = out + 8*i;
		memset(o, 0, 8*sizeof(double));
		o[0] = (double)c->kind;
		switch(c->kind){
		case JOINT_PIVOT: case JOINT_GROOVE: o[1] = c->jAcc.x; o[2] = c->jAcc.y; o[7] = c->biasv.x; break;
		case JOINT_PIN: case JOINT_SLIDE: o[1] = c->jnAcc; o[2] = c->nMass; o[7] = c->bias; break;
		case JOINT_DSPRING: o[1] = c->jnAcc; o[2] = c->nMass; o[7] = c->v_coef; break;
		case JOINT_DRSPRING: o[1] = c->jnAcc; o[2] = c->iSum; o[3] = c->w_coef; o[7] = c->target_wrn; break;
		case JOINT_RATCHET: o[1] = c->jnAcc; o[2] = c->iSum; o[3] = c->angle; o[7] = c->bias; break;
		case JOINT_ROTLIMIT: case JOINT_GEAR: o[1] = c->jnAcc; o[2] = c->iSum; o[7] = c->bias; break;
		default: o[1] = c->jnAcc; o[2] = c->iSum; break;
		}
		if(c->kind <= JOINT_DSPRING){ o[3] = c->r1.x; o[4] = c->r1.y; o[5] = c->r2.x; o[6] = c->r2.y; }
	}
	return sp->ncons;
}


/* Shape-id pairs (min, max) whose boxes intersected in the last step: the
 * pair set the broadphase handed to the narrow phase. */
int cpx_dump_candidates(cpSpace *sp, int *out, int max)
{
	int n = sp->ncand/2;
	for(int i = 0; i < n && i < max; i++){ out[2*i] = sp->candPairs[2*i]; out[2*i + 1] = sp->candPairs[2*i + 1]; }
	return n;
}

/* ========================================================================
 * Spatial queries: cpSpaceQuery.c:49-212 over the two trees (cpBBTree.c
 * SubtreeQuery :355-365, SubtreeSegmentQuery :367-385), with the shapes'
 * point and segment queries (cpShape.c:222-256, 298-318, 407-468,
 * cpPolyShape.c:66-149, chipmunk_private.h:120-142).
 * ====================================================================== */
#define ORC_MAGIC_EPSILON 1e-5

static int filter_reject_(cpShapeFilter a, cpShapeFilter b)
{
	return (a.group != 0 && a.group == b.group) || (a.categories & b.mask) == 0 || (b.categories & a.mask) == 0;
}

/* chipmunk.h:183-188 */
static cpVect closest_on_segment_(cpVect p, cpVect a, cpVect b)
{
	cpVect delta = cpvsub(a, b);
	cpFloat t = fclamp01_(cpvdot(delta, cpvsub(p, b))/cpvlengthsq(delta));
	return cpvadd(b, cpvmult(delta, t));
}

/* chipmunk_private.h:120-142 */
static void circle_segment_query_(const cpShape *shape, cpVect center, cpFloat r1, cpVect a, cpVect b, cpFloat r2, cpSegmentQueryInfo *info)
{
	cpVect da = cpvsub(a, center);
	cpVect db = cpvsub(b, center);
	cpFloat rsum = r1 + r2;
	cpFloat qa = cpvdot(da, da) - 2.0*cpvdot(da, db) + cpvdot(db, db);
	cpFloat qb = cpvdot(da, db) - cpvdot(da, da);
	cpFloat det = qb*qb - qa*(cpvdot(da, da) - rsum*rsum);
	if(det >= 0.0){
		cpFloat t = (-qb - sqrt(det))/(qa);
		if(0.0 <= t && t <= 1.0){
			cpVect n = cpvnormalize(cpvlerp(da, db, t));
			info->shape = shape;
			info->point = cpvsub(cpvlerp(a, b, t), cpvmult(n, r2));
			info->normal = n;
			info->alpha = t;
		}
	}
}

static void shape_point_query_(const cpShape *s, cpVect p, cpPointQueryInfo *info)
{
	if(s->kind == SHAPE_CIRCLE){
		/* cpShape.c:298-312 */
		cpVect delta = cpvsub(p, s->tc);
		cpFloat d = cpvlength(delta);
		cpFloat r = s->r;
		info->shape = s;
		cpFloat r_over_d = d > 0.0 ? r/d : r;
		info->point = cpvadd(s->tc, cpvmult(delta, r_over_d));
		info->distance = d - r;
		info->gradient = (d > ORC_MAGIC_EPSILON ? cpvmult(delta, 1.0/d) : cpv(0.0, 1.0));
	} else if(s->kind == SHAPE_SEGMENT){
		/* cpShape.c:407-423; the small-distance gradient is the local normal */
		cpVect closest = closest_on_segment_(p, s->ta, s->tb);
		cpVect delta = cpvsub(p, closest);
		cpFloat d = cpvlength(delta);
		cpFloat r = s->r;
		cpVect g = cpvmult(delta, 1.0/d);
		info->shape = s;
		info->point = (d ? cpvadd(closest, cpvmult(g, r)) : closest);
		info->distance = d - r;
		info->gradient = (d > ORC_MAGIC_EPSILON ? g : s->sn);
	} else {
		/* cpPolyShape.c:66-103 */
		int count = s->count;
		cpFloat r = s->r;
		cpVect v0 = s->pv[count - 1];
		cpFloat minDist = ORC_INF;
		cpVect closestPoint = cpvzero, closestNormal = cpvzero;
		cpBool outside = cpFalse;
		for(int i = 0; i < count; i++){
			cpVect v1 = s->pv[i];
			outside = outside || (cpvdot(s->pn[i], cpvsub(p, v1)) > 0.0);
			cpVect closest = closest_on_segment_(p, v0, v1);
			cpFloat dist = cpvdist(p, closest);
			if(dist < minDist){
				minDist = dist;
				closestPoint = closest;
				closestNormal = s->pn[i];
			}
			v0 = v1;
		}
		cpFloat dist = (outside ? minDist : -minDist);
		cpVect g = cpvmult(cpvsub(p, closestPoint), 1.0/dist);
		info->shape = s;
		info->point = cpvadd(closestPoint, cpvmult(g, r));
		info->distance = dist - r;
		info->gradient = (minDist > ORC_MAGIC_EPSILON ? g : closestNormal);
	}
}

static void shape_segment_query_(const cpShape *s, cpVect a, cpVect b, cpFloat r2, cpSegmentQueryInfo *info)
{
	if(s->kind == SHAPE_CIRCLE){
		circle_segment_query_(s, s->tc, s->r, a, b, r2, info);
	} else if(s->kind == SHAPE_SEGMENT){
		/* cpShape.c:425-468 */
		cpVect n = s->tn;
		cpFloat d = cpvdot(cpvsub(s->ta, a), n);
		cpFloat r = s->r + r2;
		cpVect flipped_n = (d > 0.0 ? cpvneg(n) : n);
		cpVect seg_offset = cpvsub(cpvmult(flipped_n, r), a);
		cpVect seg_a = cpvadd(s->ta, seg_offset);
		cpVect seg_b = cpvadd(s->tb, seg_offset);
		cpVect delta = cpvsub(b, a);
		if(cpvcross(delta, seg_a)*cpvcross(delta, seg_b) <= 0.0){
			cpFloat d_offset = d + (d > 0.0 ? -r : r);
			cpFloat ad = -d_offset;
			cpFloat bd = cpvdot(delta, n) - d_offset;
			if(ad*bd < 0.0){
				cpFloat t = ad/(ad - bd);
				info->shape = s;
				info->point = cpvsub(cpvlerp(a, b, t), cpvmult(flipped_n, r2));
				info->normal = flipped_n;
				info->alpha = t;
			}
		} else if(r != 0.0){
			cpSegmentQueryInfo info1 = {NULL, b, cpvzero, 1.0};
			cpSegmentQueryInfo info2 = {NULL, b, cpvzero, 1.0};
			circle_segment_query_(s, s->ta, s->r, a, b, r2, &info1);
			circle_segment_query_(s, s->tb, s->r, a, b, r2, &info2);
			if(info1.alpha < info2.alpha) *info = info1; else *info = info2;
		}
	} else {
		/* cpPolyShape.c:105-149 */
		int count = s->count;
		cpFloat r = s->r;
		cpFloat rsum = r + r2;
		for(int i = 0; i < count; i++){
			cpVect n = s->pn[i];
			cpFloat an = cpvdot(a, n);
			cpFloat d = an - cpvdot(s->pv[i], n) - rsum;
			if(d < 0.0) continue;
			cpFloat bn = cpvdot(b, n);
			cpFloat t = d/fmax_(an - bn, DBL_MIN);
			if(t < 0.0 || 1.0 < t) continue;
			cpVect point = cpvlerp(a, b, t);
			cpFloat dt = cpvcross(n, point);
			cpFloat dtMin = cpvcross(n, s->pv[(i - 1 + count)%count]);
			cpFloat dtMax = cpvcross(n, s->pv[i]);
			if(dtMin <= dt && dt <= dtMax){
				info->shape = s;
				info->point = cpvsub(cpvlerp(a, b, t), cpvmult(n, r2));
				info->normal = n;
				info->alpha = t;
			}
		}
		if(rsum > 0.0){
			for(int i = 0; i < count; i++){
				cpSegmentQueryInfo circle_info = {NULL, b, cpvzero, 1.0};
				circle_segment_query_(s, s->pv[i], r, a, b, r2, &circle_info);
				if(circle_info.alpha < info->alpha) *info = circle_info;
			}
		}
	}
}

/* cpShape.c:222-235 */
cpFloat cpShapePointQuery(const cpShape *shape, cpVect p, cpPointQueryInfo *info)
{
	cpPointQueryInfo blank = {NULL, cpvzero, ORC_INF, cpvzero};
	if(info) *info = blank; else info = &blank;
	shape_point_query_(shape, p, info);
	return info->distance;
}

/* cpShape.c:238-256 */
cpBool cpShapeSegmentQuery(const cpShape *shape, cpVect a, cpVect b, cpFloat radius, cpSegmentQueryInfo *info)
{
	cpSegmentQueryInfo blank = {NULL, b, cpvzero, 1.0};
	if(info) *info = blank; else info = &blank;
	cpPointQueryInfo nearest;
	shape_point_query_(shape, a, &nearest);
	if(nearest.distance <= radius){
		info->shape = shape;
		info->alpha = 0.0;
		info->normal = cpvnormalize(cpvsub(a, nearest.point));
	} else {
		shape_segment_query_(shape, a, b, radius, info);
	}
	return (info->shape != NULL);
}

/* cpBB.h:115-143 */
static cpFloat bb_segment_query_(cpBB bb, cpVect a, cpVect b)
{
	cpVect delta = cpvsub(b, a);
	cpFloat tmin = -ORC_INF, tmax = ORC_INF;
	if(delta.x == 0.0){
		if(a.x < bb.l || bb.r < a.x) return ORC_INF;
	} else {
		cpFloat t1 = (bb.l - a.x)/delta.x;
		cpFloat t2 = (bb.r - a.x)/delta.x;
		tmin = fmax_(tmin, fmin_(t1, t2));
		tmax = fmin_(tmax, fmax_(t1, t2));
	}
	if(delta.y == 0.0){
		if(a.y < bb.b || bb.t < a.y) return ORC_INF;
	} else {
		cpFloat t1 = (bb.b - a.y)/delta.y;
		cpFloat t2 = (bb.t - a.y)/delta.y;
		tmin = fmax_(tmin, fmin_(t1, t2));
		tmax = fmin_(tmax, fmax_(t1, t2));
	}
	if(tmin <= tmax && 0.0 <= tmax && tmin <= 1.0) return fmax_(tmin, 0.0);
	return ORC_INF;
}

typedef struct QueryCtx {
	int kind;                 /* 0 point, 1 nearest, 2 segment, 3 first, 4 box */
	cpVect a, b;
	cpFloat r;
	cpBB bb;
	cpShapeFilter filter;
	void *func, *data;
	cpPointQueryInfo *pout;
	cpSegmentQueryInfo *sout;
} QueryCtx;

/* the leaf callbacks of cpSpaceQuery.c: NearestPointQuery :33-46,
 * NearestPointQueryNearest :61-74, SegmentQuery :105-121, SegmentQueryFirst
 * :138-152 (returns the running best alpha), BBQuery :183-193 */
static cpFloat query_leaf_(QueryCtx *q, cpShape *shape)
{
	if(filter_reject_(shape->filter, q->filter)) return (q->kind == 3) ? q->sout->alpha : 1.0;
	switch(q->kind){
	case 0: {
		cpPointQueryInfo info;
		cpShapePointQuery(shape, q->a, &info);
		if(info.shape && info.distance < q->r)
			((cpSpacePointQueryFunc)q->func)(shape, info.point, info.distance, info.gradient, q->data);
		return 1.0;
	}
	case 1:
		if(!shape->sensor){
			cpPointQueryInfo info;
			cpShapePointQuery(shape, q->a, &info);
			if(info.distance < q->pout->distance) *q->pout = info;
		}
		return 1.0;
	case 2: {
		cpSegmentQueryInfo info;
		if(cpShapeSegmentQuery(shape, q->a, q->b, q->r, &info))
			((cpSpaceSegmentQueryFunc)q->func)(shape, info.point, info.normal, info.alpha, q->data);
		return 1.0;
	}
	case 3: {
		cpSegmentQueryInfo info;
		if(!shape->sensor && cpShapeSegmentQuery(shape, q->a, q->b, q->r, &info) && info.alpha < q->sout->alpha)
			*q->sout = info;
		return q->sout->alpha;
	}
	default:
		if(cpBBIntersects(q->bb, shape->bb)) ((cpSpaceBBQueryFunc)q->func)(shape, q->data);
		return 1.0;
	}
}

/* cpBBTree.c:355-365 */
static void subtree_query_(cpSpace *sp, int n, QueryCtx *q)
{
	Node *nd = &sp->nodes[n];
	if(cpBBIntersects(nd->bb, q->bb)){
		if(nd->obj) query_leaf_(q, nd->obj);
		else {
			subtree_query_(sp, nd->A, q);
			subtree_query_(sp, sp->nodes[n].B, q);
		}
	}
}

/* cpBBTree.c:367-385 */
static cpFloat subtree_segment_query_(cpSpace *sp, int n, QueryCtx *q, cpFloat t_exit)
{
	Node *nd = &sp->nodes[n];
	if(nd->obj) return query_leaf_(q, nd->obj);
	int A = nd->A, B = nd->B;
	cpFloat t_a = bb_segment_query_(sp->nodes[A].bb, q->a, q->b);
	cpFloat t_b = bb_segment_query_(sp->nodes[B].bb, q->a, q->b);
	if(t_a < t_b){
		if(t_a < t_exit) t_exit = fmin_(t_exit, subtree_segment_query_(sp, A, q, t_exit));
		if(t_b < t_exit) t_exit = fmin_(t_exit, subtree_segment_query_(sp, B, q, t_exit));
	} else {
		if(t_b < t_exit) t_exit = fmin_(t_exit, subtree_segment_query_(sp, B, q, t_exit));
		if(t_a < t_exit) t_exit = fmin_(t_exit, subtree_segment_query_(sp, A, q, t_exit));
	}
	return t_exit;
}

/* cpSpaceHashQuery (cpSpaceHash.c:353-392): the cells of the box, each
 * handle once (its stamp) */
static void hash_query_(cpSpace *sp, HashGrid *g, QueryCtx *q)
{
	cpBB bb = q->bb;
	cpFloat dim = g->celldim;
	int l = floor_int_(bb.l/dim), r = floor_int_(bb.r/dim);
	int b = floor_int_(bb.b/dim), t = floor_int_(bb.t/dim);
	for(int i = l; i <= r; i++){
		for(int j = b; j <= t; j++){
			int cell = (int)hash_cell_(i, j, g->numcells);
			for(int bn = g->cells[cell]; bn >= 0; bn = g->binNext[bn]){
				int other = g->binHandle[bn];
				if(sp->nodes[other].stamp == g->stamp) continue;
				query_leaf_(q, sp->nodes[other].obj);
				sp->nodes[other].stamp = g->stamp;
			}
		}
	}
	g->stamp++;
}

/* cpSpaceHashSegmentQuery (cpSpaceHash.c:443-525): the cells along the
 * segment in order, a grid walk */
static void hash_segment_query_(cpSpace *sp, HashGrid *g, QueryCtx *q, cpFloat t_exit)
{
	cpVect a = cpvmult(q->a, 1.0f/g->celldim), b = cpvmult(q->b, 1.0f/g->celldim);
	int cell_x = floor_int_(a.x), cell_y = floor_int_(a.y);
	cpFloat t = 0;
	int x_inc, y_inc;
	cpFloat temp_v, temp_h;
	if(b.x > a.x){ x_inc = 1; temp_h = (floor(a.x + 1.0f) - a.x); } else { x_inc = -1; temp_h = (a.x - floor(a.x)); }
	if(b.y > a.y){ y_inc = 1; temp_v = (floor(a.y + 1.0f) - a.y); } else { y_inc = -1; temp_v = (a.y - floor(a.y)); }
	cpFloat dx = fabs_(b.x - a.x), dy = fabs_(b.y - a.y);
	cpFloat dt_dx = (dx ? 1.0f/dx : ORC_INF), dt_dy = (dy ? 1.0f/dy : ORC_INF);
	cpFloat next_h = (temp_h ? temp_h*dt_dx : dt_dx);
	cpFloat next_v = (temp_v ? temp_v*dt_dy : dt_dy);
	while(t < t_exit){
		int cell = (int)hash_cell_(cell_x, cell_y, g->numcells);
		/* segmentQuery_helper (:395-418) */
		cpFloat tc = 1.0f;
		for(int bn = g->cells[cell]; bn >= 0; bn = g->binNext[bn]){
			int other = g->binHandle[bn];
			if(sp->nodes[other].stamp == g->stamp) continue;
			tc = fmin_(tc, query_leaf_(q, sp->nodes[other].obj));
			sp->nodes[other].stamp = g->stamp;
		}
		t_exit = fmin_(t_exit, tc);
		if(next_v < next_h){ cell_y += y_inc; t = next_v; next_v += dt_dy; }
		else { cell_x += x_inc; t = next_h; next_h += dt_dx; }
	}
	g->stamp++;
}

static void tree_query_(cpSpace *sp, Tree *t, QueryCtx *q)
{
	if(sp->useHash){ hash_query_(sp, t->isDynamic ? &sp->dynGrid : &sp->statGrid, q); return; }
	if(t->root >= 0) subtree_query_(sp, t->root, q);
}
static void tree_segment_query_(cpSpace *sp, Tree *t, QueryCtx *q, cpFloat t_exit)
{
	if(sp->useHash){ hash_segment_query_(sp, t->isDynamic ? &sp->dynGrid : &sp->statGrid, q, t_exit); return; }
	if(t->root >= 0) subtree_segment_query_(sp, t->root, q, t_exit);
}

/* cpSpaceQuery.c:48-57 */
void cpSpacePointQuery(cpSpace *sp, cpVect point, cpFloat maxDistance, cpShapeFilter filter, cpSpacePointQueryFunc func, void *data)
{
	QueryCtx q = {0};
	q.kind = 0; q.a = point; q.r = maxDistance; q.filter = filter; q.func = (void *)func; q.data = data;
	q.bb = cpBBNewForCircle(point, fmax_(maxDistance, 0.0));
	sp->locked++;
	tree_query_(sp, &sp->dynTree, &q);
	tree_query_(sp, &sp->statTree, &q);
	space_unlock_(sp);
	run_post_step_(sp);
}

/* cpSpaceQuery.c:76-98 */
cpShape *cpSpacePointQueryNearest(cpSpace *sp, cpVect point, cpFloat maxDistance, cpShapeFilter filter, cpPointQueryInfo *out)
{
	cpPointQueryInfo info = {NULL, cpvzero, maxDistance, cpvzero};
	if(out) *out = info; else out = &info;
	QueryCtx q = {0};
	q.kind = 1; q.a = point; q.r = maxDistance; q.filter = filter; q.pout = out;
	q.bb = cpBBNewForCircle(point, fmax_(maxDistance, 0.0));
	tree_query_(sp, &sp->dynTree, &q);
	tree_query_(sp, &sp->statTree, &q);
	return (cpShape *)out->shape;
}

/* cpSpaceQuery.c:123-136 */
void cpSpaceSegmentQuery(cpSpace *sp, cpVect start, cpVect end, cpFloat radius, cpShapeFilter filter, cpSpaceSegmentQueryFunc func, void *data)
{
	QueryCtx q = {0};
	q.kind = 2; q.a = start; q.b = end; q.r = radius; q.filter = filter; q.func = (void *)func; q.data = data;
	sp->locked++;
	tree_segment_query_(sp, &sp->statTree, &q, 1.0);
	tree_segment_query_(sp, &sp->dynTree, &q, 1.0);
	space_unlock_(sp);
	run_post_step_(sp);
}

/* cpSpaceQuery.c:154-175 */
cpShape *cpSpaceSegmentQueryFirst(cpSpace *sp, cpVect start, cpVect end, cpFloat radius, cpShapeFilter filter, cpSegmentQueryInfo *out)
{
	cpSegmentQueryInfo info = {NULL, end, cpvzero, 1.0};
	if(out) *out = info; else out = &info;
	QueryCtx q = {0};
	q.kind = 3; q.a = start; q.b = end; q.r = radius; q.filter = filter; q.sout = out;
	tree_segment_query_(sp, &sp->statTree, &q, 1.0);
	tree_segment_query_(sp, &sp->dynTree, &q, out->alpha);
	return (cpShape *)out->shape;
}

/* cpSpaceQuery.c:195-204 */
void cpSpaceBBQuery(cpSpace *sp, cpBB bb, cpShapeFilter filter, cpSpaceBBQueryFunc func, void *data)
{
	QueryCtx q = {0};
	q.kind = 4; q.bb = bb; q.filter = filter; q.func = (void *)func; q.data = data;
	sp->locked++;
	tree_query_(sp, &sp->dynTree, &q);
	tree_query_(sp, &sp->statTree, &q);
	space_unlock_(sp);
	run_post_step_(sp);
}


/* cpShape.c:258-283 */
cpContactPointSet cpShapesCollide(const cpShape *a, const cpShape *b)
{
	CollisionInfo info = collide((cpShape *)a, (cpShape *)b, 0);
	cpContactPointSet set;
	memset(&set, 0, sizeof(set));
	set.count = info.count;
	cpBool swapped = (a != info.a);
	set.normal = (swapped ? cpvneg(info.n) : info.n);
	for(int i = 0; i < info.count; i++){
		cpVect p1 = info.arr[i].r1, p2 = info.arr[i].r2;
		set.points[i].pointA = (swapped ? p2 : p1);
		set.points[i].pointB = (swapped ? p1 : p2);
		set.points[i].distance = cpvdot(cpvsub(p2, p1), set.normal);
	}
	return set;
}

typedef struct ShapeQueryCtx { cpShape *shape; cpSpaceShapeQueryFunc func; void *data; cpBool anyCollision; } ShapeQueryCtx;

/* cpSpaceQuery.c:214-228 (ShapeQuery) over cpBBTree.c:355-365 */
static void subtree_shape_query_(cpSpace *sp, int n, cpBB bb, ShapeQueryCtx *q)
{
	Node *nd = &sp->nodes[n];
	if(!cpBBIntersects(nd->bb, bb)) return;
	if(nd->obj){
		cpShape *a = q->shape, *b = nd->obj;
		if(filter_reject_(a->filter, b->filter) || a == b) return;
		cpContactPointSet set = cpShapesCollide(a, b);
		if(set.count){
			if(q->func) q->func(b, &set, q->data);
			q->anyCollision = !(a->sensor || b->sensor);
		}
	} else {
		int B = nd->B;
		subtree_shape_query_(sp, nd->A, bb, q);
		subtree_shape_query_(sp, B, bb, q);
	}
}

/* ShapeQuery over cpSpaceHashQuery (cpSpaceHash.c:353-392) */
static void hash_shape_query_(cpSpace *sp, HashGrid *g, cpBB bb, ShapeQueryCtx *q)
{
	cpFloat dim = g->celldim;
	int l = floor_int_(bb.l/dim), r = floor_int_(bb.r/dim);
	int b = floor_int_(bb.b/dim), t = floor_int_(bb.t/dim);
	for(int i = l; i <= r; i++){
		for(int j = b; j <= t; j++){
			int cell = (int)hash_cell_(i, j, g->numcells);
			for(int bn = g->cells[cell]; bn >= 0; bn = g->binNext[bn]){
				int other = g->binHandle[bn];
				cpShape *sb = sp->nodes[other].obj;
				if(sp->nodes[other].stamp == g->stamp || sb == q->shape) continue;
				cpShape *sa = q->shape;
				if(!filter_reject_(sa->filter, sb->filter)){
					cpContactPointSet set = cpShapesCollide(sa, sb);
					if(set.count){
						if(q->func) q->func(sb, &set, q->data);
						q->anyCollision = !(sa->sensor || sb->sensor);
					}
				}
				sp->nodes[other].stamp = g->stamp;
			}
		}
	}
	g->stamp++;
}

/* cpSpaceQuery.c:230-246 */
cpBool cpSpaceShapeQuery(cpSpace *sp, cpShape *shape, cpSpaceShapeQueryFunc func, void *data)
{
	cpBody *body = shape->body;
	cpBB bb = (body ? shape_update(shape, body->transform) : shape->bb);
	ShapeQueryCtx q = {shape, func, data, cpFalse};
	sp->locked++;
	if(sp->useHash){
		hash_shape_query_(sp, &sp->dynGrid, bb, &q);
		hash_shape_query_(sp, &sp->statGrid, bb, &q);
	} else {
		if(sp->dynTree.root >= 0) subtree_shape_query_(sp, sp->dynTree.root, bb, &q);
		if(sp->statTree.root >= 0) subtree_shape_query_(sp, sp->statTree.root, bb, &q);
	}
	space_unlock_(sp);
	run_post_step_(sp);
	return q.anyCollision;
}


/* ---- caller-placed objects (the *Alloc / *Init / *Destroy functions of
 * cpSpace.c, cpBody.c, cpShape.c, cpPolyShape.c and the joints): the New
 * functions' objects moved into the caller's memory; only a space's
 * static body refers back to its owner ---- */
static void *adopt_(void *mem, void *fresh, size_t bytes)
{
	if(mem && fresh) memcpy(mem, fresh, bytes);
	free(fresh);
	return mem;
}

cpSpace *cpSpaceAlloc(void) { return (cpSpace *)calloc(1, sizeof(cpSpace)); }
cpSpace *cpSpaceInit(cpSpace *sp) { adopt_(sp, cpSpaceNew(), sizeof(cpSpace)); sp->staticBody.space = sp; return sp; }
cpBody *cpBodyAlloc(void) { return (cpBody *)calloc(1, sizeof(cpBody)); }
cpBody *cpBodyInit(cpBody *b, cpFloat m, cpFloat i) { return (cpBody *)adopt_(b, cpBodyNew(m, i), sizeof(cpBody)); }
void cpBodyDestroy(cpBody *b) { (void)b; }
void cpShapeDestroy(cpShape *s) { if(s){ free(s->pv); free(s->pn); s->pv = s->pn = NULL; } }
void cpConstraintDestroy(cpConstraint *c) { (void)c; }

#define ORC_SHAPE_ALLOC(T) T *T##Alloc(void) { return (T *)calloc(1, sizeof(cpShape)); }
#define ORC_JOINT_ALLOC(T) T *T##Alloc(void) { return (T *)calloc(1, sizeof(cpConstraint)); }
ORC_SHAPE_ALLOC(cpCircleShape)
ORC_SHAPE_ALLOC(cpSegmentShape)
ORC_SHAPE_ALLOC(cpPolyShape)
ORC_JOINT_ALLOC(cpPivotJoint)
ORC_JOINT_ALLOC(cpPinJoint)
ORC_JOINT_ALLOC(cpSlideJoint)
ORC_JOINT_ALLOC(cpGrooveJoint)
ORC_JOINT_ALLOC(cpDampedSpring)
ORC_JOINT_ALLOC(cpDampedRotarySpring)
ORC_JOINT_ALLOC(cpRotaryLimitJoint)
ORC_JOINT_ALLOC(cpRatchetJoint)
ORC_JOINT_ALLOC(cpGearJoint)
ORC_JOINT_ALLOC(cpSimpleMotor)

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

/* the threaded space's names on the serial space (the oracle's checked
 * results are the serial solver's) */
cpSpace *cpHastySpaceNew(void) { return cpSpaceNew(); }
void cpHastySpaceFree(cpSpace *sp) { cpSpaceFree(sp); }
void cpHastySpaceSetThreads(cpSpace *sp, unsigned long threads) { (void)sp; (void)threads; }
unsigned long cpHastySpaceGetThreads(cpSpace *sp) { (void)sp; return 1ul; }
void cpHastySpaceStep(cpSpace *sp, cpFloat dt) { cpSpaceStep(sp, dt); }


/* cpSpaceStep.c:26-58 (cpSpaceAddPostStepCallback), 84-103 (run when the
 * space unlocks after a step, an iteration or a query) */
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

/*
 * chipmunk_gb300.h -- C ABI of the GB300 drop-in for Chipmunk2D's cpSpaceStep path.
 *
 * Every function below keeps the name, argument meaning and error behaviour of
 * the Chipmunk2D 7.0.3 public function it replaces; the comment beside each
 * group cites the reference declaration (file:line, relative to the
 * Chipmunk2D source tree).  The value types (cpVect, cpBB, cpTransform,
 * cpShapeFilter, cpContactPointSet, ...) have the reference's exact memory
 * layout, so an object file compiled against the reference headers links
 * against libchipmunk_gb300.so unchanged: every object is handled through an
 * opaque pointer and every by-value struct has the same layout.
 *
 * Functions prefixed cpGpu* have no counterpart in the reference; they are the
 * GPU-only additions (solver mode, batching, error side channel, stream and
 * debug state export).
 *
 * Threading and errors follow the reference: not thread-safe; API misuse
 * aborts through cpMessage (include/chipmunk/chipmunk.h:48-58).  Device-side
 * failures (bounded waits that timed out, table overflow) never abort; they
 * are latched and reported by cpGpuGetLastError().
 */
#ifndef CHIPMUNK_GB300_H
#define CHIPMUNK_GB300_H

#include <stdint.h>
#include <stddef.h>
#include <math.h>
#include <float.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- scalar types: include/chipmunk/chipmunk_types.h:55-67, 162-231 ---- */
typedef double cpFloat;
typedef uintptr_t cpHashValue;
typedef uint32_t cpCollisionID;
typedef unsigned char cpBool;
typedef void *cpDataPointer;
typedef uintptr_t cpCollisionType;
typedef uintptr_t cpGroup;
typedef unsigned int cpBitmask;
typedef unsigned int cpTimestamp;

#define cpTrue 1
#define cpFalse 0
#define CP_NO_GROUP ((cpGroup)0)
#define CP_ALL_CATEGORIES (~(cpBitmask)0)
#define CP_WILDCARD_COLLISION_TYPE (~(cpCollisionType)0)
#define CP_MAX_CONTACTS_PER_ARBITER 2

/* ---- value structs: chipmunk_types.h:236-266, cpBB.h:31-33 ---- */
typedef struct cpVect { cpFloat x, y; } cpVect;
typedef struct cpTransform { cpFloat a, b, c, d, tx, ty; } cpTransform;
typedef struct cpMat2x2 { cpFloat a, b, c, d; } cpMat2x2;
typedef struct cpBB { cpFloat l, b, r, t; } cpBB;

/* ---- opaque handles: chipmunk.h:85-111 ---- */
typedef struct cpBody cpBody;
typedef struct cpShape cpShape;
typedef struct cpCircleShape cpCircleShape;
typedef struct cpSegmentShape cpSegmentShape;
typedef struct cpPolyShape cpPolyShape;
typedef struct cpConstraint cpConstraint;
typedef struct cpPinJoint cpPinJoint;
typedef struct cpSlideJoint cpSlideJoint;
typedef struct cpPivotJoint cpPivotJoint;
typedef struct cpGrooveJoint cpGrooveJoint;
typedef struct cpDampedSpring cpDampedSpring;
typedef struct cpDampedRotarySpring cpDampedRotarySpring;
typedef struct cpRotaryLimitJoint cpRotaryLimitJoint;
typedef struct cpRatchetJoint cpRatchetJoint;
typedef struct cpGearJoint cpGearJoint;
typedef struct cpSimpleMotor cpSimpleMotor;
typedef struct cpArbiter cpArbiter;
typedef struct cpSpace cpSpace;
typedef struct cpCollisionHandler cpCollisionHandler;
typedef struct cpContactPointSet cpContactPointSet;

/* cpShape.h:27-58 */
typedef struct cpPointQueryInfo {
	const cpShape *shape;
	cpVect point;
	cpFloat distance;
	cpVect gradient;
} cpPointQueryInfo;

typedef struct cpSegmentQueryInfo {
	const cpShape *shape;
	cpVect point;
	cpVect normal;
	cpFloat alpha;
} cpSegmentQueryInfo;

typedef struct cpShapeFilter {
	cpGroup group;
	cpBitmask categories;
	cpBitmask mask;
} cpShapeFilter;

/* cpArbiter.h:81-96 */
struct cpContactPointSet {
	int count;
	cpVect normal;
	struct {
		cpVect pointA, pointB;
		cpFloat distance;
	} points[CP_MAX_CONTACTS_PER_ARBITER];
};

/* cpBody.h:28-46, 175-185 */
typedef enum cpBodyType {
	CP_BODY_TYPE_DYNAMIC,
	CP_BODY_TYPE_KINEMATIC,
	CP_BODY_TYPE_STATIC,
} cpBodyType;

typedef void (*cpBodyVelocityFunc)(cpBody *body, cpVect gravity, cpFloat damping, cpFloat dt);
typedef void (*cpBodyPositionFunc)(cpBody *body, cpFloat dt);
typedef void (*cpBodyShapeIteratorFunc)(cpBody *body, cpShape *shape, void *data);
typedef void (*cpBodyConstraintIteratorFunc)(cpBody *body, cpConstraint *constraint, void *data);
typedef void (*cpBodyArbiterIteratorFunc)(cpBody *body, cpArbiter *arbiter, void *data);

/* cpSpace.h:28-55, 220-236 */
typedef cpBool (*cpCollisionBeginFunc)(cpArbiter *arb, cpSpace *space, cpDataPointer userData);
typedef cpBool (*cpCollisionPreSolveFunc)(cpArbiter *arb, cpSpace *space, cpDataPointer userData);
typedef void (*cpCollisionPostSolveFunc)(cpArbiter *arb, cpSpace *space, cpDataPointer userData);
typedef void (*cpCollisionSeparateFunc)(cpArbiter *arb, cpSpace *space, cpDataPointer userData);

struct cpCollisionHandler {
	const cpCollisionType typeA;
	const cpCollisionType typeB;
	cpCollisionBeginFunc beginFunc;
	cpCollisionPreSolveFunc preSolveFunc;
	cpCollisionPostSolveFunc postSolveFunc;
	cpCollisionSeparateFunc separateFunc;
	cpDataPointer userData;
};

typedef void (*cpSpaceBodyIteratorFunc)(cpBody *body, void *data);
typedef void (*cpSpaceShapeIteratorFunc)(cpShape *shape, void *data);
typedef void (*cpSpaceConstraintIteratorFunc)(cpConstraint *constraint, void *data);

/* Query callbacks: cpSpace.h:196-210 */
typedef void (*cpSpacePointQueryFunc)(cpShape *shape, cpVect point, cpFloat distance, cpVect gradient, void *data);
typedef void (*cpSpaceSegmentQueryFunc)(cpShape *shape, cpVect point, cpVect normal, cpFloat alpha, void *data);
typedef void (*cpSpaceBBQueryFunc)(cpShape *shape, void *data);
typedef void (*cpSpaceShapeQueryFunc)(cpShape *shape, cpContactPointSet *points, void *data);
typedef void (*cpPostStepFunc)(cpSpace *space, void *key, void *data);               /* cpSpace.h:182 */

/* cpConstraint.h:25-29 */
typedef void (*cpConstraintPreSolveFunc)(cpConstraint *constraint, cpSpace *space);
typedef void (*cpConstraintPostSolveFunc)(cpConstraint *constraint, cpSpace *space);

/* ------------------------------------------------------------------------
 * Inline value helpers.  The reference ships these as static inline
 * functions (cpVect.h:35-225, cpBB.h:35-190, cpTransform.h:30-140); they
 * compile into the caller, so they are restated here for programs that use
 * this header instead of the reference's.
 * ---------------------------------------------------------------------- */
static const cpVect cpvzero = {0.0, 0.0};
static inline cpVect cpv(const cpFloat x, const cpFloat y) { cpVect v = {x, y}; return v; }
static inline cpBool cpveql(const cpVect a, const cpVect b) { return (a.x == b.x && a.y == b.y); }
static inline cpVect cpvadd(const cpVect a, const cpVect b) { return cpv(a.x + b.x, a.y + b.y); }
static inline cpVect cpvsub(const cpVect a, const cpVect b) { return cpv(a.x - b.x, a.y - b.y); }
static inline cpVect cpvneg(const cpVect a) { return cpv(-a.x, -a.y); }
static inline cpVect cpvmult(const cpVect a, const cpFloat s) { return cpv(a.x*s, a.y*s); }
static inline cpFloat cpvdot(const cpVect a, const cpVect b) { return a.x*b.x + a.y*b.y; }
static inline cpFloat cpvcross(const cpVect a, const cpVect b) { return a.x*b.y - a.y*b.x; }
static inline cpVect cpvperp(const cpVect a) { return cpv(-a.y, a.x); }
static inline cpVect cpvrperp(const cpVect a) { return cpv(a.y, -a.x); }
/* cpVect.h:98-101 */
static inline cpVect cpvproject(const cpVect v1, const cpVect v2) { return cpvmult(v2, cpvdot(v1, v2)/cpvdot(v2, v2)); }
static inline cpVect cpvrotate(const cpVect a, const cpVect b) { return cpv(a.x*b.x - a.y*b.y, a.x*b.y + a.y*b.x); }
static inline cpVect cpvunrotate(const cpVect a, const cpVect b) { return cpv(a.x*b.x + a.y*b.y, a.y*b.x - a.x*b.y); }
static inline cpFloat cpvlengthsq(const cpVect a) { return cpvdot(a, a); }
static inline cpFloat cpvlength(const cpVect a) { return sqrt(cpvdot(a, a)); }
static inline cpVect cpvlerp(const cpVect a, const cpVect b, const cpFloat t) { return cpvadd(cpvmult(a, 1.0 - t), cpvmult(b, t)); }
static inline cpVect cpvnormalize(const cpVect a) { return cpvmult(a, 1.0/(cpvlength(a) + DBL_MIN)); }
static inline cpFloat cpvdist(const cpVect a, const cpVect b) { return cpvlength(cpvsub(a, b)); }
static inline cpFloat cpvdistsq(const cpVect a, const cpVect b) { return cpvlengthsq(cpvsub(a, b)); }
static inline cpVect cpvforangle(const cpFloat a) { return cpv(cos(a), sin(a)); }
static inline cpFloat cpvtoangle(const cpVect v) { return atan2(v.y, v.x); }

static inline cpBB cpBBNew(const cpFloat l, const cpFloat b, const cpFloat r, const cpFloat t) { cpBB bb = {l, b, r, t}; return bb; }
static inline cpBB cpBBNewForExtents(const cpVect c, const cpFloat hw, const cpFloat hh) { return cpBBNew(c.x - hw, c.y - hh, c.x + hw, c.y + hh); }
static inline cpBB cpBBNewForCircle(const cpVect p, const cpFloat r) { return cpBBNewForExtents(p, r, r); }
static inline cpBool cpBBIntersects(const cpBB a, const cpBB b) { return (a.l <= b.r && b.l <= a.r && a.b <= b.t && b.b <= a.t); }
static inline cpBool cpBBContainsBB(const cpBB bb, const cpBB o) { return (bb.l <= o.l && bb.r >= o.r && bb.b <= o.b && bb.t >= o.t); }
static inline cpVect cpBBCenter(cpBB bb) { return cpvlerp(cpv(bb.l, bb.b), cpv(bb.r, bb.t), 0.5); }
static inline cpFloat cpBBArea(cpBB bb) { return (bb.r - bb.l)*(bb.t - bb.b); }

static const cpTransform cpTransformIdentity = {1.0, 0.0, 0.0, 1.0, 0.0, 0.0};
static inline cpTransform cpTransformNew(cpFloat a, cpFloat b, cpFloat c, cpFloat d, cpFloat tx, cpFloat ty) { cpTransform t = {a, b, c, d, tx, ty}; return t; }
static inline cpTransform cpTransformNewTranspose(cpFloat a, cpFloat c, cpFloat tx, cpFloat b, cpFloat d, cpFloat ty) { cpTransform t = {a, b, c, d, tx, ty}; return t; }
static inline cpVect cpTransformPoint(cpTransform t, cpVect p) { return cpv(t.a*p.x + t.c*p.y + t.tx, t.b*p.x + t.d*p.y + t.ty); }
static inline cpVect cpTransformVect(cpTransform t, cpVect v) { return cpv(t.a*v.x + t.c*v.y, t.b*v.x + t.d*v.y); }

static inline cpShapeFilter cpShapeFilterNew(cpGroup group, cpBitmask categories, cpBitmask mask) { cpShapeFilter f = {group, categories, mask}; return f; }
static const cpShapeFilter CP_SHAPE_FILTER_ALL = {CP_NO_GROUP, CP_ALL_CATEGORIES, CP_ALL_CATEGORIES};
static const cpShapeFilter CP_SHAPE_FILTER_NONE = {CP_NO_GROUP, ~CP_ALL_CATEGORIES, ~CP_ALL_CATEGORIES};

/* ------------------------------------------------------------------------
 * Misc: chipmunk.h:48, 134-171
 * ---------------------------------------------------------------------- */
void cpMessage(const char *condition, const char *file, int line, int isError, int isHardError, const char *message, ...);
extern const char *cpVersionString;
cpFloat cpMomentForCircle(cpFloat m, cpFloat r1, cpFloat r2, cpVect offset);
cpFloat cpAreaForCircle(cpFloat r1, cpFloat r2);
cpFloat cpMomentForSegment(cpFloat m, cpVect a, cpVect b, cpFloat radius);
cpFloat cpAreaForSegment(cpVect a, cpVect b, cpFloat radius);
cpFloat cpMomentForPoly(cpFloat m, int count, const cpVect *verts, cpVect offset, cpFloat radius);
cpFloat cpAreaForPoly(const int count, const cpVect *verts, cpFloat radius);
cpVect cpCentroidForPoly(const int count, const cpVect *verts);
cpFloat cpMomentForBox(cpFloat m, cpFloat width, cpFloat height);
cpFloat cpMomentForBox2(cpFloat m, cpBB box);
int cpConvexHull(int count, const cpVect *verts, cpVect *result, int *first, cpFloat tol);

/* ------------------------------------------------------------------------
 * Space: cpSpace.h:68-255
 * ---------------------------------------------------------------------- */
cpSpace *cpSpaceNew(void);                                           /* cpSpace.h:72  */
void cpSpaceFree(cpSpace *space);                                    /* cpSpace.h:77  */
int cpSpaceGetIterations(const cpSpace *space);                      /* cpSpace.h:83  */
void cpSpaceSetIterations(cpSpace *space, int iterations);           /* cpSpace.h:84  */
cpVect cpSpaceGetGravity(const cpSpace *space);                      /* cpSpace.h:87  */
void cpSpaceSetGravity(cpSpace *space, cpVect gravity);              /* cpSpace.h:88  */
cpFloat cpSpaceGetDamping(const cpSpace *space);                     /* cpSpace.h:94  */
void cpSpaceSetDamping(cpSpace *space, cpFloat damping);             /* cpSpace.h:95  */
cpFloat cpSpaceGetIdleSpeedThreshold(const cpSpace *space);          /* cpSpace.h:99  */
void cpSpaceSetIdleSpeedThreshold(cpSpace *space, cpFloat v);        /* cpSpace.h:100 */
cpFloat cpSpaceGetSleepTimeThreshold(const cpSpace *space);          /* cpSpace.h:105 */
void cpSpaceSetSleepTimeThreshold(cpSpace *space, cpFloat t);        /* cpSpace.h:106 */
cpFloat cpSpaceGetCollisionSlop(const cpSpace *space);               /* cpSpace.h:112 */
void cpSpaceSetCollisionSlop(cpSpace *space, cpFloat slop);          /* cpSpace.h:113 */
cpFloat cpSpaceGetCollisionBias(const cpSpace *space);               /* cpSpace.h:118 */
void cpSpaceSetCollisionBias(cpSpace *space, cpFloat bias);          /* cpSpace.h:119 */
cpTimestamp cpSpaceGetCollisionPersistence(const cpSpace *space);    /* cpSpace.h:123 */
void cpSpaceSetCollisionPersistence(cpSpace *space, cpTimestamp n);  /* cpSpace.h:124 */
cpDataPointer cpSpaceGetUserData(const cpSpace *space);              /* cpSpace.h:129 */
void cpSpaceSetUserData(cpSpace *space, cpDataPointer userData);     /* cpSpace.h:130 */
cpBody *cpSpaceGetStaticBody(const cpSpace *space);                  /* cpSpace.h:134 */
cpFloat cpSpaceGetCurrentTimeStep(const cpSpace *space);             /* cpSpace.h:138 */
cpBool cpSpaceIsLocked(cpSpace *space);                              /* cpSpace.h:141 */
cpShape *cpSpaceAddShape(cpSpace *space, cpShape *shape);            /* cpSpace.h:159 */
cpBody *cpSpaceAddBody(cpSpace *space, cpBody *body);                /* cpSpace.h:161 */
cpConstraint *cpSpaceAddConstraint(cpSpace *space, cpConstraint *c); /* cpSpace.h:163 */
/* Removal (and addition) between steps: the next cpSpaceStep rebuilds the
 * device set, carrying the tree, pair cache and arbiter cache over, and
 * replays the index edits in call order; removal order follows the
 * reference's arrays (the last element takes the hole). */
void cpSpaceRemoveShape(cpSpace *space, cpShape *shape);              /* cpSpace.h:166 */
void cpSpaceRemoveBody(cpSpace *space, cpBody *body);                 /* cpSpace.h:168 */
void cpSpaceRemoveConstraint(cpSpace *space, cpConstraint *constraint); /* cpSpace.h:170 */
cpBool cpSpaceContainsShape(cpSpace *space, cpShape *shape);         /* cpSpace.h:173 */
cpBool cpSpaceContainsBody(cpSpace *space, cpBody *body);            /* cpSpace.h:175 */
cpBool cpSpaceContainsConstraint(cpSpace *space, cpConstraint *c);   /* cpSpace.h:177 */
void cpSpaceEachBody(cpSpace *space, cpSpaceBodyIteratorFunc func, void *data);             /* cpSpace.h:226 */
void cpSpaceEachShape(cpSpace *space, cpSpaceShapeIteratorFunc func, void *data);           /* cpSpace.h:231 */
void cpSpaceEachConstraint(cpSpace *space, cpSpaceConstraintIteratorFunc func, void *data); /* cpSpace.h:236 */
void cpSpaceStep(cpSpace *space, cpFloat dt);                        /* cpSpace.h:255 */
/* Re-indexing moved shapes (cpSpace.h:240-246): the caches are brought to
 * the bodies' transforms at the call and the trees updated as the
 * reference's are, before the next step or query. */
void cpSpaceReindexStatic(cpSpace *space);                           /* cpSpace.h:240 */
/* The spatial hash as both indices (cpSpace.h:249): the broadphase then
 * visits pairs in the hash's order, as the reference's does. */
void cpSpaceUseSpatialHash(cpSpace *space, cpFloat dim, int count);   /* cpSpace.h:249 */
void cpSpaceReindexShape(cpSpace *space, cpShape *shape);            /* cpSpace.h:242 */
void cpSpaceReindexShapesForBody(cpSpace *space, cpBody *body);      /* cpSpace.h:244 */
/* A callback run once when the current (or next) step, body/shape/
 * constraint iteration or point/segment/box/shape query ends, one per key;
 * returns cpFalse when the key is already registered. */
cpBool cpSpaceAddPostStepCallback(cpSpace *space, cpPostStepFunc func, void *key, void *data);     /* cpSpace.h:187 */
/* Caller-placed objects (cpSpace.h:80-88, cpBody.h:49-58, cpShape.h:78-84,
 * 161-197, cpPolyShape.h:26-40, cpConstraint.h:61, the joints' headers):
 * cp*Alloc returns zeroed memory of the object's size, cp*Init
 * initialises it as the matching cp*New does and returns it, cp*Destroy
 * releases what an object holds without freeing the object itself. */
cpSpace *cpSpaceAlloc(void);
cpSpace *cpSpaceInit(cpSpace *space);
void cpSpaceDestroy(cpSpace *space);
cpBody *cpBodyAlloc(void);
cpBody *cpBodyInit(cpBody *body, cpFloat mass, cpFloat moment);
void cpBodyDestroy(cpBody *body);
void cpShapeDestroy(cpShape *shape);
cpCircleShape *cpCircleShapeAlloc(void);
cpCircleShape *cpCircleShapeInit(cpCircleShape *circle, cpBody *body, cpFloat radius, cpVect offset);
cpSegmentShape *cpSegmentShapeAlloc(void);
cpSegmentShape *cpSegmentShapeInit(cpSegmentShape *seg, cpBody *body, cpVect a, cpVect b, cpFloat radius);
cpPolyShape *cpPolyShapeAlloc(void);
cpPolyShape *cpPolyShapeInit(cpPolyShape *poly, cpBody *body, int count, const cpVect *verts, cpTransform transform, cpFloat radius);
cpPolyShape *cpPolyShapeInitRaw(cpPolyShape *poly, cpBody *body, int count, const cpVect *verts, cpFloat radius);
cpPolyShape *cpBoxShapeInit(cpPolyShape *poly, cpBody *body, cpFloat width, cpFloat height, cpFloat radius);
cpPolyShape *cpBoxShapeInit2(cpPolyShape *poly, cpBody *body, cpBB box, cpFloat radius);
void cpConstraintDestroy(cpConstraint *constraint);
cpPivotJoint *cpPivotJointAlloc(void);
cpPivotJoint *cpPivotJointInit(cpPivotJoint *joint, cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB);
cpPinJoint *cpPinJointAlloc(void);
cpPinJoint *cpPinJointInit(cpPinJoint *joint, cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB);
cpSlideJoint *cpSlideJointAlloc(void);
cpSlideJoint *cpSlideJointInit(cpSlideJoint *joint, cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB, cpFloat min, cpFloat max);
cpGrooveJoint *cpGrooveJointAlloc(void);
cpGrooveJoint *cpGrooveJointInit(cpGrooveJoint *joint, cpBody *a, cpBody *b, cpVect groove_a, cpVect groove_b, cpVect anchorB);
cpDampedSpring *cpDampedSpringAlloc(void);
cpDampedSpring *cpDampedSpringInit(cpDampedSpring *joint, cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB,
                                   cpFloat restLength, cpFloat stiffness, cpFloat damping);
cpDampedRotarySpring *cpDampedRotarySpringAlloc(void);
cpDampedRotarySpring *cpDampedRotarySpringInit(cpDampedRotarySpring *joint, cpBody *a, cpBody *b, cpFloat restAngle,
                                               cpFloat stiffness, cpFloat damping);
cpRotaryLimitJoint *cpRotaryLimitJointAlloc(void);
cpRotaryLimitJoint *cpRotaryLimitJointInit(cpRotaryLimitJoint *joint, cpBody *a, cpBody *b, cpFloat min, cpFloat max);
cpRatchetJoint *cpRatchetJointAlloc(void);
cpRatchetJoint *cpRatchetJointInit(cpRatchetJoint *joint, cpBody *a, cpBody *b, cpFloat phase, cpFloat ratchet);
cpGearJoint *cpGearJointAlloc(void);
cpGearJoint *cpGearJointInit(cpGearJoint *joint, cpBody *a, cpBody *b, cpFloat phase, cpFloat ratio);
cpSimpleMotor *cpSimpleMotorAlloc(void);
cpSimpleMotor *cpSimpleMotorInit(cpSimpleMotor *joint, cpBody *a, cpBody *b, cpFloat rate);

/* cpHastySpace.h:6-27: the threaded space's entry points.  The device
 * step is the solver here, so a hasty space is a space; the thread count
 * is kept and reported. */
cpSpace *cpHastySpaceNew(void);
void cpHastySpaceFree(cpSpace *space);
void cpHastySpaceSetThreads(cpSpace *space, unsigned long threads);
unsigned long cpHastySpaceGetThreads(cpSpace *space);
void cpHastySpaceStep(cpSpace *space, cpFloat dt);

/* Spatial queries (cpSpaceQuery.c:49-212).  They run on the device, over
 * the space's own trees in the exact-order mode (the reference's visit
 * order: dynamic then static shapes for point and box queries, static
 * then dynamic for segment queries), and the callbacks are then called
 * on the host in that order.  Objects added or removed since the last
 * step are indexed first.  In the coloured mode the dynamic tree is not
 * kept current, so every shape is tested and callbacks come in the
 * space's shape order. */
void cpSpacePointQuery(cpSpace *space, cpVect point, cpFloat maxDistance, cpShapeFilter filter,
                       cpSpacePointQueryFunc func, void *data);                                    /* cpSpace.h:198 */
cpShape *cpSpacePointQueryNearest(cpSpace *space, cpVect point, cpFloat maxDistance, cpShapeFilter filter,
                                  cpPointQueryInfo *out);                                          /* cpSpace.h:200 */
void cpSpaceSegmentQuery(cpSpace *space, cpVect start, cpVect end, cpFloat radius, cpShapeFilter filter,
                         cpSpaceSegmentQueryFunc func, void *data);                                /* cpSpace.h:205 */
cpShape *cpSpaceSegmentQueryFirst(cpSpace *space, cpVect start, cpVect end, cpFloat radius, cpShapeFilter filter,
                                  cpSegmentQueryInfo *out);                                        /* cpSpace.h:207 */
void cpSpaceBBQuery(cpSpace *space, cpBB bb, cpShapeFilter filter, cpSpaceBBQueryFunc func, void *data); /* cpSpace.h:212 */
/* Shapes overlapping a shape (cpSpaceQuery.c:214-246): its cache is
 * brought to its body's transform, as the reference does, and each
 * overlapping shape comes with its contact point set. */
cpBool cpSpaceShapeQuery(cpSpace *space, cpShape *shape, cpSpaceShapeQueryFunc func, void *data);     /* cpSpace.h:217 */

/* ------------------------------------------------------------------------
 * Body: cpBody.h:49-187
 * ---------------------------------------------------------------------- */
cpBody *cpBodyNew(cpFloat mass, cpFloat moment);                     /* cpBody.h:53  */
cpBody *cpBodyNewKinematic(void);                                    /* cpBody.h:56  */
cpBody *cpBodyNewStatic(void);                                       /* cpBody.h:58  */
void cpBodyFree(cpBody *body);                                       /* cpBody.h:63  */
void cpBodyActivate(cpBody *body);                                   /* cpBody.h:67  */
void cpBodyActivateStatic(cpBody *body, cpShape *filter);            /* cpBody.h:69  */
void cpBodySleep(cpBody *body);                                      /* cpBody.h:72  */
void cpBodySleepWithGroup(cpBody *body, cpBody *group);              /* cpBody.h:74  */
cpBool cpBodyIsSleeping(const cpBody *body);                         /* cpBody.h:77  */
cpBodyType cpBodyGetType(cpBody *body);                              /* cpBody.h:80  */
void cpBodySetType(cpBody *body, cpBodyType type);                    /* cpBody.h:82  */
cpSpace *cpBodyGetSpace(const cpBody *body);                         /* cpBody.h:85  */
cpFloat cpBodyGetMass(const cpBody *body);                           /* cpBody.h:88  */
void cpBodySetMass(cpBody *body, cpFloat m);                         /* cpBody.h:90  */
cpFloat cpBodyGetMoment(const cpBody *body);                         /* cpBody.h:93  */
void cpBodySetMoment(cpBody *body, cpFloat i);                       /* cpBody.h:95  */
cpVect cpBodyGetPosition(const cpBody *body);                        /* cpBody.h:98  */
void cpBodySetPosition(cpBody *body, cpVect pos);                    /* cpBody.h:100 */
cpVect cpBodyGetCenterOfGravity(const cpBody *body);                 /* cpBody.h:103 */
void cpBodySetCenterOfGravity(cpBody *body, cpVect cog);             /* cpBody.h:105 */
cpVect cpBodyGetVelocity(const cpBody *body);                        /* cpBody.h:108 */
void cpBodySetVelocity(cpBody *body, cpVect velocity);               /* cpBody.h:110 */
cpVect cpBodyGetForce(const cpBody *body);                           /* cpBody.h:113 */
void cpBodySetForce(cpBody *body, cpVect force);                     /* cpBody.h:115 */
cpFloat cpBodyGetAngle(const cpBody *body);                          /* cpBody.h:118 */
void cpBodySetAngle(cpBody *body, cpFloat a);                        /* cpBody.h:120 */
cpFloat cpBodyGetAngularVelocity(const cpBody *body);                /* cpBody.h:123 */
void cpBodySetAngularVelocity(cpBody *body, cpFloat w);              /* cpBody.h:125 */
cpFloat cpBodyGetTorque(const cpBody *body);                         /* cpBody.h:128 */
void cpBodySetTorque(cpBody *body, cpFloat torque);                  /* cpBody.h:130 */
cpVect cpBodyGetRotation(const cpBody *body);                        /* cpBody.h:133 */
cpDataPointer cpBodyGetUserData(const cpBody *body);                 /* cpBody.h:136 */
void cpBodySetUserData(cpBody *body, cpDataPointer userData);        /* cpBody.h:138 */
void cpBodySetVelocityUpdateFunc(cpBody *body, cpBodyVelocityFunc f);/* cpBody.h:141 */
void cpBodySetPositionUpdateFunc(cpBody *body, cpBodyPositionFunc f);/* cpBody.h:144 */
void cpBodyUpdateVelocity(cpBody *body, cpVect gravity, cpFloat damping, cpFloat dt); /* cpBody.h:147 */
void cpBodyUpdatePosition(cpBody *body, cpFloat dt);                 /* cpBody.h:149 */
cpVect cpBodyLocalToWorld(const cpBody *body, const cpVect point);   /* cpBody.h:152 */
cpVect cpBodyWorldToLocal(const cpBody *body, const cpVect point);   /* cpBody.h:154 */
void cpBodyApplyForceAtWorldPoint(cpBody *body, cpVect force, cpVect point);     /* cpBody.h:157 */
void cpBodyApplyForceAtLocalPoint(cpBody *body, cpVect force, cpVect point);     /* cpBody.h:159 */
void cpBodyApplyImpulseAtWorldPoint(cpBody *body, cpVect impulse, cpVect point); /* cpBody.h:162 */
void cpBodyApplyImpulseAtLocalPoint(cpBody *body, cpVect impulse, cpVect point); /* cpBody.h:164 */
cpVect cpBodyGetVelocityAtWorldPoint(const cpBody *body, cpVect point);          /* cpBody.h:167 */
cpVect cpBodyGetVelocityAtLocalPoint(const cpBody *body, cpVect point);          /* cpBody.h:169 */
cpFloat cpBodyKineticEnergy(const cpBody *body);                                 /* cpBody.h:172 */
void cpBodyEachShape(cpBody *body, cpBodyShapeIteratorFunc func, void *data);    /* cpBody.h:177 */
void cpBodyEachConstraint(cpBody *body, cpBodyConstraintIteratorFunc func, void *data); /* cpBody.h:182 */
void cpBodyEachArbiter(cpBody *body, cpBodyArbiterIteratorFunc func, void *data);       /* cpBody.h:187 */

/* ------------------------------------------------------------------------
 * Shapes: cpShape.h:78-197, cpPolyShape.h:26-54
 * ---------------------------------------------------------------------- */
void cpShapeFree(cpShape *shape);                                    /* cpShape.h:80  */
cpBB cpShapeCacheBB(cpShape *shape);                                 /* cpShape.h:83  */
cpBB cpShapeUpdate(cpShape *shape, cpTransform transform);           /* cpShape.h:85  */
void cpShapeSetBody(cpShape *shape, cpBody *body);                   /* cpShape.h:104 */
cpSpace *cpShapeGetSpace(const cpShape *shape);                      /* cpShape.h:98  */
cpBody *cpShapeGetBody(const cpShape *shape);                        /* cpShape.h:101 */
cpFloat cpShapeGetMass(cpShape *shape);                              /* cpShape.h:107 */
void cpShapeSetMass(cpShape *shape, cpFloat mass);                   /* cpShape.h:109 */
cpFloat cpShapeGetDensity(cpShape *shape);                           /* cpShape.h:112 */
void cpShapeSetDensity(cpShape *shape, cpFloat density);             /* cpShape.h:114 */
cpFloat cpShapeGetMoment(cpShape *shape);                            /* cpShape.h:117 */
cpFloat cpShapeGetArea(cpShape *shape);                              /* cpShape.h:119 */
cpVect cpShapeGetCenterOfGravity(cpShape *shape);                    /* cpShape.h:121 */
cpBB cpShapeGetBB(const cpShape *shape);                             /* cpShape.h:124 */
cpBool cpShapeGetSensor(const cpShape *shape);                       /* cpShape.h:127 */
void cpShapeSetSensor(cpShape *shape, cpBool sensor);                /* cpShape.h:129 */
cpFloat cpShapeGetElasticity(const cpShape *shape);                  /* cpShape.h:132 */
void cpShapeSetElasticity(cpShape *shape, cpFloat elasticity);       /* cpShape.h:134 */
cpFloat cpShapeGetFriction(const cpShape *shape);                    /* cpShape.h:137 */
void cpShapeSetFriction(cpShape *shape, cpFloat friction);           /* cpShape.h:139 */
cpVect cpShapeGetSurfaceVelocity(const cpShape *shape);              /* cpShape.h:142 */
void cpShapeSetSurfaceVelocity(cpShape *shape, cpVect v);            /* cpShape.h:144 */
cpDataPointer cpShapeGetUserData(const cpShape *shape);              /* cpShape.h:147 */
void cpShapeSetUserData(cpShape *shape, cpDataPointer userData);     /* cpShape.h:149 */
cpCollisionType cpShapeGetCollisionType(const cpShape *shape);       /* cpShape.h:152 */
void cpShapeSetCollisionType(cpShape *shape, cpCollisionType t);     /* cpShape.h:154 */
cpShapeFilter cpShapeGetFilter(const cpShape *shape);                /* cpShape.h:157 */
void cpShapeSetFilter(cpShape *shape, cpShapeFilter filter);         /* cpShape.h:159 */
/* One shape against a point or a segment, on its world geometry of the
 * last step (cpShape.c:222-256). */
cpFloat cpShapePointQuery(const cpShape *shape, cpVect p, cpPointQueryInfo *out);                  /* cpShape.h:89 */
cpBool cpShapeSegmentQuery(const cpShape *shape, cpVect a, cpVect b, cpFloat radius, cpSegmentQueryInfo *info); /* cpShape.h:92 */
/* The contact points of two shapes at their cached positions (cpShape.c:258-283). */
cpContactPointSet cpShapesCollide(const cpShape *a, const cpShape *b);                              /* cpShape.h:95 */
cpShape *cpCircleShapeNew(cpBody *body, cpFloat radius, cpVect offset);      /* cpShape.h:170 */
cpVect cpCircleShapeGetOffset(const cpShape *shape);                         /* cpShape.h:173 */
cpFloat cpCircleShapeGetRadius(const cpShape *shape);                        /* cpShape.h:175 */
cpShape *cpSegmentShapeNew(cpBody *body, cpVect a, cpVect b, cpFloat radius);/* cpShape.h:185 */
void cpSegmentShapeSetNeighbors(cpShape *shape, cpVect prev, cpVect next);   /* cpShape.h:188 */

/* chipmunk_unsafe.h:47-63: shapes changed in place (the space's set is
 * rebuilt with the new geometry before its next step) */
void cpCircleShapeSetRadius(cpShape *shape, cpFloat radius);         /* chipmunk_unsafe.h:47 */
void cpCircleShapeSetOffset(cpShape *shape, cpVect offset);          /* chipmunk_unsafe.h:49 */
void cpSegmentShapeSetEndpoints(cpShape *shape, cpVect a, cpVect b); /* chipmunk_unsafe.h:52 */
void cpSegmentShapeSetRadius(cpShape *shape, cpFloat radius);        /* chipmunk_unsafe.h:54 */
void cpPolyShapeSetVerts(cpShape *shape, int count, cpVect *verts, cpTransform transform); /* chipmunk_unsafe.h:57 */
void cpPolyShapeSetVertsRaw(cpShape *shape, int count, cpVect *verts); /* chipmunk_unsafe.h:58 */
void cpPolyShapeSetRadius(cpShape *shape, cpFloat radius);           /* chipmunk_unsafe.h:60 */
cpVect cpSegmentShapeGetA(const cpShape *shape);                             /* cpShape.h:191 */
cpVect cpSegmentShapeGetB(const cpShape *shape);                             /* cpShape.h:193 */
cpVect cpSegmentShapeGetNormal(const cpShape *shape);                        /* cpShape.h:195 */
cpFloat cpSegmentShapeGetRadius(const cpShape *shape);                       /* cpShape.h:197 */
cpShape *cpPolyShapeNew(cpBody *body, int count, const cpVect *verts, cpTransform transform, cpFloat radius); /* cpPolyShape.h:35 */
cpShape *cpPolyShapeNewRaw(cpBody *body, int count, const cpVect *verts, cpFloat radius);                    /* cpPolyShape.h:38 */
cpShape *cpBoxShapeNew(cpBody *body, cpFloat width, cpFloat height, cpFloat radius);                         /* cpPolyShape.h:45 */
cpShape *cpBoxShapeNew2(cpBody *body, cpBB box, cpFloat radius);                                             /* cpPolyShape.h:47 */
int cpPolyShapeGetCount(const cpShape *shape);                               /* cpPolyShape.h:50 */
cpVect cpPolyShapeGetVert(const cpShape *shape, int index);                  /* cpPolyShape.h:52 */
cpFloat cpPolyShapeGetRadius(const cpShape *shape);                          /* cpPolyShape.h:54 */

/* ------------------------------------------------------------------------
 * Constraints: cpConstraint.h:31-82, cpPivotJoint.h:26-45,
 * cpPinJoint.h:26-48, cpSlideJoint.h:26-53
 * ---------------------------------------------------------------------- */
void cpConstraintFree(cpConstraint *constraint);                             /* cpConstraint.h:33 */
cpSpace *cpConstraintGetSpace(const cpConstraint *constraint);               /* cpConstraint.h:36 */
cpBody *cpConstraintGetBodyA(const cpConstraint *constraint);                /* cpConstraint.h:39 */
cpBody *cpConstraintGetBodyB(const cpConstraint *constraint);                /* cpConstraint.h:42 */
cpFloat cpConstraintGetMaxForce(const cpConstraint *constraint);             /* cpConstraint.h:45 */
void cpConstraintSetMaxForce(cpConstraint *constraint, cpFloat maxForce);    /* cpConstraint.h:47 */
cpFloat cpConstraintGetErrorBias(const cpConstraint *constraint);            /* cpConstraint.h:50 */
void cpConstraintSetErrorBias(cpConstraint *constraint, cpFloat errorBias);  /* cpConstraint.h:54 */
cpFloat cpConstraintGetMaxBias(const cpConstraint *constraint);              /* cpConstraint.h:57 */
void cpConstraintSetMaxBias(cpConstraint *constraint, cpFloat maxBias);      /* cpConstraint.h:59 */
cpBool cpConstraintGetCollideBodies(const cpConstraint *constraint);         /* cpConstraint.h:62 */
void cpConstraintSetCollideBodies(cpConstraint *constraint, cpBool collideBodies); /* cpConstraint.h:64 */
void cpConstraintSetPreSolveFunc(cpConstraint *constraint, cpConstraintPreSolveFunc f);   /* cpConstraint.h:69 */
cpConstraintPreSolveFunc cpConstraintGetPreSolveFunc(const cpConstraint *constraint);     /* cpConstraint.h:67 */
cpConstraintPostSolveFunc cpConstraintGetPostSolveFunc(const cpConstraint *constraint);   /* cpConstraint.h:72 */
void cpConstraintSetPostSolveFunc(cpConstraint *constraint, cpConstraintPostSolveFunc f); /* cpConstraint.h:74 */
cpDataPointer cpConstraintGetUserData(const cpConstraint *constraint);       /* cpConstraint.h:77 */
void cpConstraintSetUserData(cpConstraint *constraint, cpDataPointer data);  /* cpConstraint.h:79 */
cpFloat cpConstraintGetImpulse(cpConstraint *constraint);                    /* cpConstraint.h:82 */

cpBool cpConstraintIsPivotJoint(const cpConstraint *constraint);             /* cpPivotJoint.h:26 */
cpConstraint *cpPivotJointNew(cpBody *a, cpBody *b, cpVect pivot);           /* cpPivotJoint.h:33 */
cpConstraint *cpPivotJointNew2(cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB); /* cpPivotJoint.h:35 */
cpVect cpPivotJointGetAnchorA(const cpConstraint *constraint);               /* cpPivotJoint.h:38 */
cpVect cpPivotJointGetAnchorB(const cpConstraint *constraint);               /* cpPivotJoint.h:43 */
void cpPivotJointSetAnchorA(cpConstraint *constraint, cpVect anchorA);       /* cpPivotJoint.h:40 */
void cpPivotJointSetAnchorB(cpConstraint *constraint, cpVect anchorB);       /* cpPivotJoint.h:45 */

cpBool cpConstraintIsPinJoint(const cpConstraint *constraint);               /* cpPinJoint.h:26 */
cpConstraint *cpPinJointNew(cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB);    /* cpPinJoint.h:33 */
cpVect cpPinJointGetAnchorA(const cpConstraint *constraint);                 /* cpPinJoint.h:36 */
cpVect cpPinJointGetAnchorB(const cpConstraint *constraint);                 /* cpPinJoint.h:41 */
cpFloat cpPinJointGetDist(const cpConstraint *constraint);                   /* cpPinJoint.h:46 */
void cpPinJointSetAnchorA(cpConstraint *constraint, cpVect anchorA);         /* cpPinJoint.h:38 */
void cpPinJointSetAnchorB(cpConstraint *constraint, cpVect anchorB);         /* cpPinJoint.h:43 */
void cpPinJointSetDist(cpConstraint *constraint, cpFloat dist);              /* cpPinJoint.h:48 */

cpBool cpConstraintIsSlideJoint(const cpConstraint *constraint);             /* cpSlideJoint.h:26 */
cpConstraint *cpSlideJointNew(cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB, cpFloat min, cpFloat max); /* cpSlideJoint.h:33 */
cpVect cpSlideJointGetAnchorA(const cpConstraint *constraint);               /* cpSlideJoint.h:36 */
cpVect cpSlideJointGetAnchorB(const cpConstraint *constraint);               /* cpSlideJoint.h:41 */
cpFloat cpSlideJointGetMin(const cpConstraint *constraint);                  /* cpSlideJoint.h:46 */
cpFloat cpSlideJointGetMax(const cpConstraint *constraint);                  /* cpSlideJoint.h:51 */
void cpSlideJointSetAnchorA(cpConstraint *constraint, cpVect anchorA);       /* cpSlideJoint.h:38 */
void cpSlideJointSetAnchorB(cpConstraint *constraint, cpVect anchorB);       /* cpSlideJoint.h:43 */
void cpSlideJointSetMin(cpConstraint *constraint, cpFloat min);              /* cpSlideJoint.h:48 */
void cpSlideJointSetMax(cpConstraint *constraint, cpFloat max);              /* cpSlideJoint.h:53 */

/* The remaining joints: cpGrooveJoint.h, cpDampedSpring.h,
 * cpDampedRotarySpring.h, cpRotaryLimitJoint.h, cpRatchetJoint.h,
 * cpGearJoint.h, cpSimpleMotor.h.  A space whose spring uses a force or
 * torque function other than the default is refused at the step
 * (CP_GPU_ERR_UNSUPPORTED): callbacks are host code. */
typedef cpFloat (*cpDampedSpringForceFunc)(cpConstraint *spring, cpFloat dist);                 /* cpDampedSpring.h:29 */
typedef cpFloat (*cpDampedRotarySpringTorqueFunc)(cpConstraint *spring, cpFloat relativeAngle); /* cpDampedRotarySpring.h:29 */
cpBool cpConstraintIsGrooveJoint(const cpConstraint *constraint);            /* cpGrooveJoint.h:26 */
cpConstraint *cpGrooveJointNew(cpBody *a, cpBody *b, cpVect groove_a, cpVect groove_b, cpVect anchorB); /* cpGrooveJoint.h:33 */
cpVect cpGrooveJointGetGrooveA(const cpConstraint *constraint);              /* cpGrooveJoint.h:36 */
void cpGrooveJointSetGrooveA(cpConstraint *constraint, cpVect grooveA);      /* cpGrooveJoint.h:38 */
cpVect cpGrooveJointGetGrooveB(const cpConstraint *constraint);              /* cpGrooveJoint.h:41 */
void cpGrooveJointSetGrooveB(cpConstraint *constraint, cpVect grooveB);      /* cpGrooveJoint.h:43 */
cpVect cpGrooveJointGetAnchorB(const cpConstraint *constraint);              /* cpGrooveJoint.h:46 */
void cpGrooveJointSetAnchorB(cpConstraint *constraint, cpVect anchorB);      /* cpGrooveJoint.h:48 */
cpBool cpConstraintIsDampedSpring(const cpConstraint *constraint);           /* cpDampedSpring.h:26 */
cpConstraint *cpDampedSpringNew(cpBody *a, cpBody *b, cpVect anchorA, cpVect anchorB, cpFloat restLength, cpFloat stiffness, cpFloat damping); /* cpDampedSpring.h:36 */
cpVect cpDampedSpringGetAnchorA(const cpConstraint *constraint);             /* cpDampedSpring.h:39 */
void cpDampedSpringSetAnchorA(cpConstraint *constraint, cpVect anchorA);     /* cpDampedSpring.h:41 */
cpVect cpDampedSpringGetAnchorB(const cpConstraint *constraint);             /* cpDampedSpring.h:44 */
void cpDampedSpringSetAnchorB(cpConstraint *constraint, cpVect anchorB);     /* cpDampedSpring.h:46 */
cpFloat cpDampedSpringGetRestLength(const cpConstraint *constraint);         /* cpDampedSpring.h:49 */
void cpDampedSpringSetRestLength(cpConstraint *constraint, cpFloat restLength); /* cpDampedSpring.h:51 */
cpFloat cpDampedSpringGetStiffness(const cpConstraint *constraint);          /* cpDampedSpring.h:54 */
void cpDampedSpringSetStiffness(cpConstraint *constraint, cpFloat stiffness); /* cpDampedSpring.h:56 */
cpFloat cpDampedSpringGetDamping(const cpConstraint *constraint);            /* cpDampedSpring.h:59 */
void cpDampedSpringSetDamping(cpConstraint *constraint, cpFloat damping);    /* cpDampedSpring.h:61 */
cpDampedSpringForceFunc cpDampedSpringGetSpringForceFunc(const cpConstraint *constraint);               /* cpDampedSpring.h:64 */
void cpDampedSpringSetSpringForceFunc(cpConstraint *constraint, cpDampedSpringForceFunc springForceFunc); /* cpDampedSpring.h:66 */
cpBool cpConstraintIsDampedRotarySpring(const cpConstraint *constraint);     /* cpDampedRotarySpring.h:26 */
cpConstraint *cpDampedRotarySpringNew(cpBody *a, cpBody *b, cpFloat restAngle, cpFloat stiffness, cpFloat damping); /* cpDampedRotarySpring.h:36 */
cpFloat cpDampedRotarySpringGetRestAngle(const cpConstraint *constraint);    /* cpDampedRotarySpring.h:39 */
void cpDampedRotarySpringSetRestAngle(cpConstraint *constraint, cpFloat restAngle); /* cpDampedRotarySpring.h:41 */
cpFloat cpDampedRotarySpringGetStiffness(const cpConstraint *constraint);    /* cpDampedRotarySpring.h:44 */
void cpDampedRotarySpringSetStiffness(cpConstraint *constraint, cpFloat stiffness); /* cpDampedRotarySpring.h:46 */
cpFloat cpDampedRotarySpringGetDamping(const cpConstraint *constraint);      /* cpDampedRotarySpring.h:49 */
void cpDampedRotarySpringSetDamping(cpConstraint *constraint, cpFloat damping); /* cpDampedRotarySpring.h:51 */
cpDampedRotarySpringTorqueFunc cpDampedRotarySpringGetSpringTorqueFunc(const cpConstraint *constraint);                /* cpDampedRotarySpring.h:54 */
void cpDampedRotarySpringSetSpringTorqueFunc(cpConstraint *constraint, cpDampedRotarySpringTorqueFunc springTorqueFunc); /* cpDampedRotarySpring.h:56 */
cpBool cpConstraintIsRotaryLimitJoint(const cpConstraint *constraint);       /* cpRotaryLimitJoint.h:26 */
cpConstraint *cpRotaryLimitJointNew(cpBody *a, cpBody *b, cpFloat min, cpFloat max); /* cpRotaryLimitJoint.h:33 */
cpFloat cpRotaryLimitJointGetMin(const cpConstraint *constraint);            /* cpRotaryLimitJoint.h:36 */
void cpRotaryLimitJointSetMin(cpConstraint *constraint, cpFloat min);        /* cpRotaryLimitJoint.h:38 */
cpFloat cpRotaryLimitJointGetMax(const cpConstraint *constraint);            /* cpRotaryLimitJoint.h:41 */
void cpRotaryLimitJointSetMax(cpConstraint *constraint, cpFloat max);        /* cpRotaryLimitJoint.h:43 */
cpBool cpConstraintIsRatchetJoint(const cpConstraint *constraint);           /* cpRatchetJoint.h:26 */
cpConstraint *cpRatchetJointNew(cpBody *a, cpBody *b, cpFloat phase, cpFloat ratchet); /* cpRatchetJoint.h:33 */
cpFloat cpRatchetJointGetAngle(const cpConstraint *constraint);              /* cpRatchetJoint.h:36 */
void cpRatchetJointSetAngle(cpConstraint *constraint, cpFloat angle);        /* cpRatchetJoint.h:38 */
cpFloat cpRatchetJointGetPhase(const cpConstraint *constraint);              /* cpRatchetJoint.h:41 */
void cpRatchetJointSetPhase(cpConstraint *constraint, cpFloat phase);        /* cpRatchetJoint.h:43 */
cpFloat cpRatchetJointGetRatchet(const cpConstraint *constraint);            /* cpRatchetJoint.h:46 */
void cpRatchetJointSetRatchet(cpConstraint *constraint, cpFloat ratchet);    /* cpRatchetJoint.h:48 */
cpBool cpConstraintIsGearJoint(const cpConstraint *constraint);              /* cpGearJoint.h:26 */
cpConstraint *cpGearJointNew(cpBody *a, cpBody *b, cpFloat phase, cpFloat ratio); /* cpGearJoint.h:33 */
cpFloat cpGearJointGetPhase(const cpConstraint *constraint);                 /* cpGearJoint.h:36 */
void cpGearJointSetPhase(cpConstraint *constraint, cpFloat phase);           /* cpGearJoint.h:38 */
cpFloat cpGearJointGetRatio(const cpConstraint *constraint);                 /* cpGearJoint.h:41 */
void cpGearJointSetRatio(cpConstraint *constraint, cpFloat ratio);           /* cpGearJoint.h:43 */
cpBool cpConstraintIsSimpleMotor(const cpConstraint *constraint);            /* cpSimpleMotor.h:29 */
cpConstraint *cpSimpleMotorNew(cpBody *a, cpBody *b, cpFloat rate);          /* cpSimpleMotor.h:36 */
cpFloat cpSimpleMotorGetRate(const cpConstraint *constraint);                /* cpSimpleMotor.h:39 */
void cpSimpleMotorSetRate(cpConstraint *constraint, cpFloat rate);           /* cpSimpleMotor.h:41 */

/* ------------------------------------------------------------------------
 * Arbiters: cpArbiter.h:32-119.  Arbiter handles are valid from the
 * cpBodyEachArbiter callback until the next cpSpaceStep, as in the reference.
 * ---------------------------------------------------------------------- */
cpFloat cpArbiterGetRestitution(const cpArbiter *arb);               /* cpArbiter.h:32  */
cpFloat cpArbiterGetFriction(const cpArbiter *arb);                  /* cpArbiter.h:36  */
cpVect cpArbiterGetSurfaceVelocity(cpArbiter *arb);                  /* cpArbiter.h:41  */
cpVect cpArbiterTotalImpulse(const cpArbiter *arb);                  /* cpArbiter.h:55  */
cpFloat cpArbiterTotalKE(const cpArbiter *arb);                      /* cpArbiter.h:58  */
void cpArbiterGetShapes(const cpArbiter *arb, cpShape **a, cpShape **b); /* cpArbiter.h:67 */
void cpArbiterGetBodies(const cpArbiter *arb, cpBody **a, cpBody **b);   /* cpArbiter.h:75 */
cpContactPointSet cpArbiterGetContactPointSet(const cpArbiter *arb); /* cpArbiter.h:99  */
cpBool cpArbiterIsFirstContact(const cpArbiter *arb);                /* cpArbiter.h:106 */
int cpArbiterGetCount(const cpArbiter *arb);                         /* cpArbiter.h:111 */
cpVect cpArbiterGetNormal(const cpArbiter *arb);                     /* cpArbiter.h:113 */
cpVect cpArbiterGetPointA(const cpArbiter *arb, int i);              /* cpArbiter.h:115 */
cpVect cpArbiterGetPointB(const cpArbiter *arb, int i);              /* cpArbiter.h:117 */
cpFloat cpArbiterGetDepth(const cpArbiter *arb, int i);              /* cpArbiter.h:119 */

/* Inside collision-handler callbacks (cpArbiter.h:34-143, cpSpace.h:144-152).
 * The callbacks run on the host between the halves of the device step, in
 * the reference's order; the arbiter's changes go back to the device. */
void cpArbiterSetRestitution(cpArbiter *arb, cpFloat restitution);   /* cpArbiter.h:34  */
void cpArbiterSetFriction(cpArbiter *arb, cpFloat friction);         /* cpArbiter.h:38  */
void cpArbiterSetSurfaceVelocity(cpArbiter *arb, cpVect vr);         /* cpArbiter.h:45  */
cpDataPointer cpArbiterGetUserData(const cpArbiter *arb);            /* cpArbiter.h:48  */
void cpArbiterSetUserData(cpArbiter *arb, cpDataPointer userData);   /* cpArbiter.h:51  */
cpBool cpArbiterIgnore(cpArbiter *arb);                              /* cpArbiter.h:62  */
void cpArbiterSetContactPointSet(cpArbiter *arb, cpContactPointSet *set); /* cpArbiter.h:103 */
cpBool cpArbiterIsRemoval(const cpArbiter *arb);                     /* cpArbiter.h:108 */
cpBool cpArbiterCallWildcardBeginA(cpArbiter *arb, cpSpace *space);  /* cpArbiter.h:123 */
cpBool cpArbiterCallWildcardBeginB(cpArbiter *arb, cpSpace *space);  /* cpArbiter.h:126 */
cpBool cpArbiterCallWildcardPreSolveA(cpArbiter *arb, cpSpace *space); /* cpArbiter.h:130 */
cpBool cpArbiterCallWildcardPreSolveB(cpArbiter *arb, cpSpace *space); /* cpArbiter.h:133 */
void cpArbiterCallWildcardPostSolveA(cpArbiter *arb, cpSpace *space); /* cpArbiter.h:136 */
void cpArbiterCallWildcardPostSolveB(cpArbiter *arb, cpSpace *space); /* cpArbiter.h:138 */
void cpArbiterCallWildcardSeparateA(cpArbiter *arb, cpSpace *space); /* cpArbiter.h:141 */
void cpArbiterCallWildcardSeparateB(cpArbiter *arb, cpSpace *space); /* cpArbiter.h:143 */
cpCollisionHandler *cpSpaceAddDefaultCollisionHandler(cpSpace *space); /* cpSpace.h:147 */
cpCollisionHandler *cpSpaceAddCollisionHandler(cpSpace *space, cpCollisionType a, cpCollisionType b); /* cpSpace.h:150 */
cpCollisionHandler *cpSpaceAddWildcardHandler(cpSpace *space, cpCollisionType type); /* cpSpace.h:152 */

/* ------------------------------------------------------------------------
 * GPU-only additions (no counterpart in the reference).
 * ---------------------------------------------------------------------- */

/* Solver mode for a space.  ORDERED sweeps arbiters and constraints in the
 * exact sequence cpSpaceStep uses (bit-compatible results); COLORED runs
 * graph-coloured Gauss-Seidel over a device sweep-and-prune pair set, which
 * is faster for large spaces but changes the sweep order. */
typedef enum cpGpuSolverMode {
	CP_GPU_SOLVER_ORDERED = 0,
	CP_GPU_SOLVER_COLORED = 1,
} cpGpuSolverMode;

/* Error codes returned by cpGpuGetLastError(). */
enum {
	CP_GPU_OK = 0,
	CP_GPU_ERR_CUDA = 1,          /* a CUDA runtime call failed */
	CP_GPU_ERR_OVERFLOW = 2,      /* a device table or list ran out of room */
	CP_GPU_ERR_UNSUPPORTED = 3,   /* the space uses a feature the GPU step does not run */
	CP_GPU_ERR_TIMEOUT = 4,       /* a bounded device wait gave up */
	CP_GPU_ERR_NO_DEVICE = 5,     /* no CUDA device is visible */
	CP_GPU_ERR_ARGUMENT = 6,      /* invalid argument to a cpGpu* entry point */
};

void cpGpuSetSolverMode(cpSpace *space, int mode);
int cpGpuGetSolverMode(const cpSpace *space);
/* Returns and clears the last device-side error (CP_GPU_* code). */
int cpGpuGetLastError(void);
/* Human-readable description of the last error. */
const char *cpGpuGetLastErrorString(void);
/* Launch all of this library's work on the given cudaStream_t (NULL = the
 * library's own stream).  Call before the first cpSpaceStep. */
void cpGpuSetStream(void *cudaStream);
/* Wait for all queued device work of the space; then host getters are free. */
void cpGpuSpaceSync(cpSpace *space);

/* Batched stepping: spaces added to a batch are stepped together, one
 * persistent launch per phase for all of them.  Every space keeps its own
 * parameters and its exact reference sweep order. */
typedef struct cpGpuBatch cpGpuBatch;
cpGpuBatch *cpGpuBatchNew(void);
void cpGpuBatchFree(cpGpuBatch *batch);
int cpGpuBatchAddSpace(cpGpuBatch *batch, cpSpace *space);
/* Step every space of the batch `steps` times with time step dt.  With
 * use_graph != 0 the per-step launches are captured once in a CUDA graph
 * and replayed (captured again when a launch argument changes).  Batches of
 * 152 or more spaces tune their launch shapes online: on a window of 12
 * steps every 256 (the first at step 32, once the scene has contacts)
 * candidate solve block sizes and tree staging choices run on interleaved
 * steps and the fastest is kept.  All candidates give the same results. */
int cpGpuBatchStep(cpGpuBatch *batch, cpFloat dt, int steps, int use_graph);
/* The tuner's choice: [0] solve block size (0 before the first window),
 * [1] tree staging (-1 automatic, 0 off).  Returns the count written. */
int cpGpuBatchGetTuning(cpGpuBatch *batch, int *out);
/* 0 turns the online tuner off (defaults are used), 1 (default) on. */
void cpGpuSetAutotune(int on);

/* Solver quality (no reference counterpart): from the space's current
 * state, the next step of time dt is run once per iteration count k = 1 ..
 * maxIters with solver `mode` (CP_GPU_SOLVER_*), and after each run out[3k-3
 * .. 3k-1] receive the RMS over all contacts of the normal residual
 * (|vn + bounce| where the accumulated normal impulse is positive, else the
 * approach speed), the RMS friction residual (|vt| inside the friction
 * cone, else slip along the friction impulse) and the largest penetration
 * (the deepest contact's overlap along its normal after the next position
 * update, from the velocities and bias velocities the solve left).  The
 * space's state is
 * restored afterwards.  Needs a standalone space stepped at least once;
 * returns 0 or -1 (with cpGpuGetLastError() set). */
int cpGpuSolverQuality(cpSpace *space, int mode, cpFloat dt, int maxIters, double *out);

/* Every dynamic body's public state in one read (the results of a step
 * without a getter call per value): 8 doubles per body, in the order the
 * bodies were added -- position (cpBodyGetPosition), velocity, angle,
 * angular velocity, rotation (cpBodyGetRotation) -- the getters' values
 * bit for bit.  After a step they are gathered on the device and copied
 * in one transfer.  Returns the number of bodies written (at most max),
 * or -1 (error set). */
int cpGpuSpaceGetBodyStates(cpSpace *space, double *out, int max);

/* Saved states.  cpGpuSpaceSaveState copies a standalone space's whole
 * simulation state on the device (bodies, shape caches, trees and pair
 * caches, arbiters with their contacts and impulses, joints with their
 * accumulated impulses, the timestamp and last dt); a later
 * cpGpuSpaceRestoreState puts it back, and steps from there repeat the
 * steps from the save bit for bit.  Restoring is refused
 * (CP_GPU_ERR_UNSUPPORTED) once objects were added, removed or edited
 * through a setter since the save; stepping, queries, reads and the
 * space's own settings (gravity, iterations, ...) are not part of it.
 * Returns NULL (error set) when the copy could not be made. */
typedef struct cpGpuSpaceState cpGpuSpaceState;
cpGpuSpaceState *cpGpuSpaceSaveState(cpSpace *space);
int cpGpuSpaceRestoreState(cpSpace *space, const cpGpuSpaceState *state);
void cpGpuSpaceStateFree(cpGpuSpaceState *state);

/* Many queries against one space in one device launch, one thread each:
 * the nearest shape within maxDistance of each point
 * (cpSpacePointQueryNearest for every point) and the first shape hit by
 * each segment (cpSpaceSegmentQueryFirst for every start/end pair).  Host
 * arrays of n entries; out[i] is what the single query returns in its
 * info argument.  Returns CP_GPU_OK or an error code. */
int cpGpuSpacePointQueryNearestBatch(cpSpace *space, int n, const cpVect *points, cpFloat maxDistance,
                                     cpShapeFilter filter, cpPointQueryInfo *out);
int cpGpuSpaceSegmentQueryFirstBatch(cpSpace *space, int n, const cpVect *starts, const cpVect *ends, cpFloat radius,
                                     cpShapeFilter filter, cpSegmentQueryInfo *out);

/* Exact-order parallel schedule of a sequential sweep.  Unit u of the
 * sweep touches dynamic bodies bodyA[u] and bodyB[u] (a negative index or
 * one >= nbodies means "no dynamic body").  On return, order[levelStart[l]
 * .. levelStart[l+1]) lists the units of level l in sweep order, and
 * *nlevels is the number of levels.  Units of one level share no body, and
 * running the levels in turn applies every body's updates in the original
 * sweep order, so the result equals the serial sweep exactly.  All pointers
 * are device pointers; levelStart holds nunits + 1 ints and must be given
 * even when nunits is 0 (levelStart[0] is always written); order and the
 * body arrays may be NULL only when nunits is 0.  The call is
 * stream-ordered on `stream` and returns a CP_GPU_* code; its scratch comes
 * from cudaMallocAsync on that stream. */
int cpGpuSolveSchedule(const int *bodyA, const int *bodyB, int nunits, int nbodies,
                       int *levelStart, int *order, int *nlevels, void *stream);

/* Same schedule as cpGpuSolveSchedule, for callers that cannot allocate
 * device memory at the time of the call (a frame loop with a fixed time
 * budget, or a host application whose memory manager owns every device
 * allocation).  No counterpart in the reference.  It allocates nothing: its
 * scratch is a fixed 8 MiB device array inside the library, present on
 * every GPU that loads the library until exit.  Limits: nunits <= 1048576
 * and nbodies <= 1048576; larger inputs are rejected with
 * CP_GPU_ERR_ARGUMENT and a message on stderr.  The first call on a device
 * does a one-time set-up with that device current: it looks up the array's
 * device address, and with CUDA's default lazy module loading that lookup
 * is also what loads this part of the library onto the device, which is
 * when the 8 MiB array is created (an allocation by the driver, and it may
 * synchronise).  So make the first call during start-up, before any frame
 * loop and before any stream capture on that device (a call with nunits =
 * 0 and a one-int levelStart does it), or run the process with
 * CUDA_MODULE_LOADING=EAGER.  Every later call allocates nothing.  The
 * cached address belongs to the device's primary context: after
 * cudaDeviceReset the library must be reloaded.  Calls share the array:
 * calls that overlap on the GPU race, so serialise them (one stream, or
 * events).  Inputs and outputs are caller-provided device pointers, as for
 * cpGpuSolveSchedule, with the same argument rules. */
int cpGpuSolveScheduleNoAlloc(const int *bodyA, const int *bodyB, int nunits, int nbodies,
                              int *levelStart, int *order, int *nlevels, void *stream);

/* Debug/state export used by the parity tests.  Layouts are fixed:
 *   bodies:      18 doubles per dynamic body, in space order:
 *                p.x p.y v.x v.y a w f.x f.y t vb.x vb.y wb tf.a tf.b tf.c tf.d tf.tx tf.ty
 *   arbiters:    34 doubles per arbiter, in solve order:
 *                hashidA hashidB count state n.x n.y e u svr.x svr.y, then per
 *                contact slot (2): r1.x r1.y r2.x r2.y nMass tMass bounce jnAcc jtAcc jBias bias hash
 *   constraints: 8 doubles per constraint, in space order:
 *                kind j0 j1 r1.x r1.y r2.x r2.y bias0
 * Each returns the number of records available (writes at most max). */
int cpGpuDebugBodies(cpSpace *space, double *out, int max);
int cpGpuDebugArbiters(cpSpace *space, double *out, int max);
int cpGpuDebugConstraints(cpSpace *space, double *out, int max);
/* Overwrite the dynamic bodies' state (same 18-double layout) and the
 * constraints' accumulated impulses; used to run one step from a state
 * taken from another implementation. */
int cpGpuDebugSetBodies(cpSpace *space, const double *in, int count);
/* Overwrite the warm-start state the next step starts from: the
 * accumulated contact impulses of the arbiters of the last solve list (in
 * the arbiters layout above, in solve order; records whose shape pair
 * differs from the listed arbiter's are skipped) and the constraints'
 * accumulated impulses (constraints layout, j0 and j1 of pivots, j0 of
 * pin and slide joints).  Returns the number of skipped arbiter records.
 * Used with cpGpuDebugSetBodies to run one step from another
 * implementation's complete state. */
int cpGpuDebugSetImpulses(cpSpace *space, const double *arbs, int narb, const double *cons, int ncons);
/* The last step's candidates in traversal order, 4 ints each: the two
 * shapes as the query passed them, the GJK feature id passed in (the pair
 * cache's) and the one the narrow phase returned. */
int cpGpuDebugNarrowIds(cpSpace *space, int *out, int max);
/* Shape-id pairs (min, max) of the last step whose boxes intersect: the
 * pair set the broadphase handed to the narrow phase (2 ints per pair). */
int cpGpuDebugCandidates(cpSpace *space, int *out, int max);

/* Per-phase device time of the last step of the space, in milliseconds,
 * measured with CUDA events on the launching stream (0 when timing is off).
 * Phases: 0 integrate+cache, 1 broadphase, 2 narrowphase, 3 arbiters,
 * 4 schedule, 5 prestep+warmstart, 6 solve. */
/* Differentiable rollout of a batch (reference-order solver).
 * cpGpuRolloutForward steps every space of the batch `steps` times by dt
 * from its current state, keeping a copy of the device state every
 * `checkpoint` steps.  cpGpuRolloutBackward then returns the gradients of
 * a scalar loss L of the final state, given dL/dp (2 per dynamic body, in
 * batch order: spaces in the order they were added, each space's dynamic
 * bodies in the order they were added), with respect to the initial
 * velocities (dLdv0: 2 per dynamic body), initial angular velocities
 * (dLdw0: 1 per dynamic body), masses (dLdm; the moment of inertia held
 * fixed, as cpBodySetMass does), and each shape's elasticity and friction
 * (dLde, dLdu: 1 per shape, all shapes of each space in order).  Any output
 * pointer may be NULL.  The forward records, per segment of `checkpoint`
 * steps, the solver's inputs (rows, levels, poses, velocities, geometry);
 * the backward recomputes each segment's solver iterations from them (a
 * segment whose recording did not fit is replayed from its checkpoint) and
 * runs the reverse steps on the device; the batch is left in the state the
 * forward ended in.  The reverse pass needs the reference-order solver
 * and one iteration count for all spaces.  Constraints and external forces are not
 * differentiated.  Returns 0 on success, -1 with cpGpuGetLastError() set. */
int cpGpuRolloutForward(cpGpuBatch *batch, cpFloat dt, int steps, int checkpoint);
int cpGpuRolloutBackward(cpGpuBatch *batch, const cpFloat *dLdp, cpFloat *dLdv0, cpFloat *dLdw0,
	cpFloat *dLdm, cpFloat *dLde, cpFloat *dLdu);
/* The general form: the loss's gradient with respect to the final
 * positions (dLdp, 2 per dynamic body), angles (dLda, 1), velocities
 * (dLdv, 2) and angular velocities (dLdw, 1) in; its gradient with respect
 * to the initial positions (dLdp0), angles (dLda0), velocities (dLdv0),
 * angular velocities (dLdw0), masses (dLdm) and each shape's elasticity
 * and friction (dLde, dLdu) out.  Any pointer may be NULL (an absent seed
 * is zero).  cpGpuRolloutBackward(b, dLdp, ...) is this call with only the
 * position seed. */
int cpGpuRolloutBackwardFull(cpGpuBatch *batch, const cpFloat *dLdp, const cpFloat *dLda, const cpFloat *dLdv, const cpFloat *dLdw,
	cpFloat *dLdp0, cpFloat *dLda0, cpFloat *dLdv0, cpFloat *dLdw0, cpFloat *dLdm, cpFloat *dLde, cpFloat *dLdu);
/* Debug: [0], [1] device milliseconds of the last cpGpuRolloutBackward
 * taken with cpGpuSetTiming(1) (replays with recording, reverse steps);
 * [2] bytes of the segment tape, [3] bytes of the checkpoints.  Returns the
 * number of values written (4), or 0. */
int cpGpuDebugRolloutTimes(cpGpuBatch *batch, double *out);
/* Debug: 0 makes cpGpuRolloutForward record nothing, so that the reverse
 * pass replays every segment from its checkpoint; 1 (the default) records.
 * Both give the same gradients. */
void cpGpuDebugSetRolloutRecording(int on);
void cpGpuSetTiming(int enabled);
/* Debug: 1 makes single-world sets always solve with the whole-grid
 * kernel (a grid barrier between levels), 0 restores the automatic choice
 * (whole grid when a world's levels average at least 64 units and it has
 * at least 2048).  Both give the same results; the parity tests use this
 * to cover the whole-grid path on small worlds. */
void cpGpuDebugSetWholeGridSolve(int always);
/* Debug: the ordered tree step keeps the node pools of worlds of at most
 * maxNodes nodes in shared memory (-1: every world whose pool fits). */
void cpGpuDebugSetTreeStaging(int maxNodes);
/* Debug: block size of the per-world solve (32, 64, 128, 256 or 512; anything
 * else restores the default) and the largest world (in bodies) whose
 * bodies it keeps in shared memory (-1: every world that fits). */
void cpGpuDebugSetSolveShape(int threads, int maxBodies);
/* Debug: lane layout of the per-world solve's levels: 0 automatic, 1 the
 * fewest FP64 warp instructions, 2 the shortest dependent chain, 3 four
 * lanes per contact only.  All give the same results. */
void cpGpuDebugSetSolveLayout(int policy);
/* Debug: the coloured mode's sweep by dataflow (1: each unit waits for the
 * units before it on its two bodies) or with a grid barrier after every
 * colour (0, default: faster on this part).  Both give the same results. */
void cpGpuDebugSetFlowSolve(int on);
/* Debug: the coloured mode's warm start (the sweep's first pass) as a
 * per-body gather of the cached impulses in colour order (1) or as colour
 * levels of the sweep (0, default).  Both give the same results. */
void cpGpuDebugSetWarmStartGather(int on);
/* Debug, tests of the bounded waits: the coloured dataflow sweep's waits
 * give up after `polls` polls (0: the default, 2^20) and then latch an
 * error that cpGpuGetLastError() reports as CP_GPU_ERR_TIMEOUT; with
 * `withhold` set the sweep publishes no completions, so every wait that
 * has a predecessor runs out (the step's results are then not defined). */
void cpGpuDebugSetFlowWaitLimit(int polls, int withhold);
/* Debug, tests of the overflow latches: capacities of the sets built from
 * now on -- candidate pairs per world (pairsPerShape * shapes +
 * pairsExtra), arbiter table slots (rounded up to a power of two) and tree
 * nodes per world; 0 (or -1 for pairsExtra) keeps a default.  A table that
 * runs out latches an error that cpGpuGetLastError() reports as
 * CP_GPU_ERR_OVERFLOW; nothing is written past it. */
void cpGpuDebugSetCapacities(int pairsPerShape, int pairsExtra, int arbiterSlots, int nodes);
/* Debug: how a single space's exact-order tree is marked: by parallel
 * phases (1), by one device thread (0), or automatically (-1, default:
 * parallel from 1024 dynamic shapes up).  All give the same candidates,
 * pair lists and results. */
void cpGpuDebugSetParallelMarking(int on);
void cpGpuDebugSetCoopBlocks(int n);
/* Bookkeeping of the last step (after it completes): [0] error flags,
 * [1] pair-pool use and [2] node-pool use (per mille of capacity, largest
 * world), [3] live cached arbiters, [4] candidate pairs, [5] solved
 * arbiters, [6] levels (ordered) or colours (coloured) of one sweep,
 * [7] candidate-buffer use (per mille), [8] leaves reinserted in the
 * exact-order tree (all worlds).  Returns the count written. */
int cpGpuGetStepStats(cpSpace *space, int *out, int max);
int cpGpuGetPhaseTimes(cpSpace *space, double *ms, int max);
/* Number of kernel launches issued by this library since the last reset. */
long long cpGpuGetLaunchCount(int reset);

#ifdef __cplusplus
}
#endif

#endif /* CHIPMUNK_GB300_H */

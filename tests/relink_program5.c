/*
 * relink_program5.c -- an ordinary Chipmunk2D program (reference public API
 * only) built on collision handlers: a one-way platform (pre-solve ignores
 * contacts from below), ball-ground contacts that count begins and
 * separations, keep a per-arbiter counter in the arbiter's user data, nudge
 * the contact points and sum the impulses after the solve; boxes that
 * refuse their first touch with a ball (begin returns false: ignored until
 * they separate); a sensor that counts what passes through it; wildcard
 * handlers for boxes that change the friction and surface velocity; the
 * default handler summing contact counts and kinetic energy; and a shape
 * removed while it touches (a separation that is a removal), with sleeping
 * on.  It prints the counters, the sums and every body's state.  Built like
 * relink_program.c.
 */
#include <stdio.h>
#include <stdlib.h>
#ifdef RELINK_REFERENCE_HEADERS
#include "chipmunk/chipmunk.h"
#else
#include "chipmunk_gb300.h"
#endif

enum { GROUND = 1, PLATFORM = 2, BOX = 3, BALL = 4, SENSOR = 5 };
#define MAXB 64

static cpBody *bodies[MAXB];
static cpShape *shapes[MAXB];
static int nbodies = 0;

static int beginBallGround, sepBallGround, removalSeps, beginBoxBall, refusedBoxBall, sepBoxBall;
static int sensorIn, sensorOut, platformIgnored, platformKept, wildBegins, wildSeps, postCount;
static long defaultContacts;
static cpVect impulseSum;
static cpFloat keSum;

static cpBool ball_ground_begin(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)space; (void)data;
	beginBallGround++;
	cpArbiterSetUserData(arb, (cpDataPointer)(size_t)1);
	return cpTrue;
}

static cpBool ball_ground_pre(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)space; (void)data;
	size_t n = (size_t)cpArbiterGetUserData(arb);
	cpArbiterSetUserData(arb, (cpDataPointer)(n + 1));
	/* lift the contact points on the ground side a little */
	cpContactPointSet set = cpArbiterGetContactPointSet(arb);
	for(int i = 0; i < set.count; i++) set.points[i].pointB = cpvadd(set.points[i].pointB, cpv(0.0, 0.01));
	cpArbiterSetContactPointSet(arb, &set);
	cpArbiterSetRestitution(arb, 0.5);
	return cpTrue;
}

static void ball_ground_post(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)space; (void)data;
	impulseSum = cpvadd(impulseSum, cpArbiterTotalImpulse(arb));
	postCount++;
}

static void ball_ground_separate(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)space; (void)data;
	sepBallGround++;
	if(cpArbiterIsRemoval(arb)) removalSeps++;
}

static cpBool platform_pre(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)space; (void)data;
	/* the box is shape a and the normal points from it to the platform:
	 * pass through when the box comes from below */
	if(cpvdot(cpArbiterGetNormal(arb), cpv(0.0, 1.0)) > 0.0){
		platformIgnored++;
		return cpArbiterIgnore(arb);
	}
	platformKept++;
	cpArbiterSetFriction(arb, 0.2);
	return cpTrue;
}

static cpBool box_ball_begin(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)space; (void)data;
	beginBoxBall++;
	cpShape *a, *b;
	cpArbiterGetShapes(arb, &a, &b);
	/* every other box lets the first touch of a ball through */
	if(((size_t)cpShapeGetUserData(a)) % 2 == 0){ refusedBoxBall++; return cpFalse; }
	return cpTrue;
}

static void box_ball_separate(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)arb; (void)space; (void)data;
	sepBoxBall++;
}

static cpBool sensor_begin(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)arb; (void)space; (void)data;
	sensorIn++;
	return cpTrue;
}

static void sensor_separate(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)arb; (void)space; (void)data;
	sensorOut++;
}

static cpBool box_wild_begin(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)space; (void)data;
	wildBegins++;
	cpArbiterSetSurfaceVelocity(arb, cpv(3.0, 0.0));
	return cpTrue;
}

static cpBool box_wild_pre(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)space; (void)data;
	cpArbiterSetFriction(arb, cpArbiterGetFriction(arb)*0.9);
	return cpTrue;
}

static void box_wild_separate(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)arb; (void)space; (void)data;
	wildSeps++;
}

static void default_post(cpArbiter *arb, cpSpace *space, cpDataPointer data)
{
	(void)data;
	defaultContacts += cpArbiterGetCount(arb);
	keSum += cpArbiterTotalKE(arb);
	cpArbiterCallWildcardPostSolveA(arb, space);
	cpArbiterCallWildcardPostSolveB(arb, space);
}

static void on_ground(cpBody *body, cpArbiter *arb, void *data)
{
	(void)body;
	cpShape *a, *b;
	cpArbiterGetShapes(arb, &a, &b);
	if(cpShapeGetCollisionType(a) == GROUND || cpShapeGetCollisionType(b) == GROUND) *(int *)data = 1;
}

static int add_box(cpSpace *space, cpVect p, cpFloat w, cpFloat h)
{
	cpBody *b = cpSpaceAddBody(space, cpBodyNew(1.0, cpMomentForBox(1.0, w, h)));
	cpBodySetPosition(b, p);
	cpShape *s = cpSpaceAddShape(space, cpBoxShapeNew(b, w, h, 0.0));
	cpShapeSetFriction(s, 0.7);
	cpShapeSetCollisionType(s, BOX);
	cpShapeSetUserData(s, (cpDataPointer)(size_t)nbodies);
	bodies[nbodies] = b; shapes[nbodies] = s;
	return nbodies++;
}

static int add_ball(cpSpace *space, cpVect p, cpFloat r, cpVect v)
{
	cpBody *b = cpSpaceAddBody(space, cpBodyNew(1.0, cpMomentForCircle(1.0, 0.0, r, cpvzero)));
	cpBodySetPosition(b, p);
	cpBodySetVelocity(b, v);
	cpShape *s = cpSpaceAddShape(space, cpCircleShapeNew(b, r, cpvzero));
	cpShapeSetFriction(s, 0.6);
	cpShapeSetElasticity(s, 0.3);
	cpShapeSetCollisionType(s, BALL);
	cpShapeSetUserData(s, (cpDataPointer)(size_t)nbodies);
	bodies[nbodies] = b; shapes[nbodies] = s;
	return nbodies++;
}

int main(void)
{
	cpSpace *space = cpSpaceNew();
	cpSpaceSetIterations(space, 10);
	cpSpaceSetGravity(space, cpv(0.0, -100.0));
	/* resting piles fall asleep; the handlers see them wake */
	cpSpaceSetSleepTimeThreshold(space, 0.5);

	cpBody *sb = cpSpaceGetStaticBody(space);
	cpShape *ground = cpSpaceAddShape(space, cpSegmentShapeNew(sb, cpv(-300.0, 0.0), cpv(300.0, 0.0), 0.0));
	cpShapeSetFriction(ground, 1.0);
	cpShapeSetElasticity(ground, 0.5);
	cpShapeSetCollisionType(ground, GROUND);
	cpShape *platform = cpSpaceAddShape(space, cpSegmentShapeNew(sb, cpv(-60.0, 40.0), cpv(60.0, 40.0), 2.0));
	cpShapeSetFriction(platform, 1.0);
	cpShapeSetCollisionType(platform, PLATFORM);
	cpShape *sensor = cpSpaceAddShape(space, cpBoxShapeNew2(sb, cpBBNew(120.0, 0.0, 160.0, 60.0), 0.0));
	cpShapeSetSensor(sensor, cpTrue);
	cpShapeSetCollisionType(sensor, SENSOR);

	cpCollisionHandler *h;
	h = cpSpaceAddCollisionHandler(space, BALL, GROUND);
	h->beginFunc = ball_ground_begin; h->preSolveFunc = ball_ground_pre;
	h->postSolveFunc = ball_ground_post; h->separateFunc = ball_ground_separate;
	h = cpSpaceAddCollisionHandler(space, BOX, PLATFORM);
	h->preSolveFunc = platform_pre;
	h = cpSpaceAddCollisionHandler(space, BALL, BOX);
	h->beginFunc = box_ball_begin; h->separateFunc = box_ball_separate;
	h = cpSpaceAddCollisionHandler(space, SENSOR, BALL);
	h->beginFunc = sensor_begin; h->separateFunc = sensor_separate;
	h = cpSpaceAddWildcardHandler(space, BOX);
	h->beginFunc = box_wild_begin; h->preSolveFunc = box_wild_pre; h->separateFunc = box_wild_separate;
	h = cpSpaceAddDefaultCollisionHandler(space);
	h->postSolveFunc = default_post;

	/* boxes launched up through the platform, some landing on it */
	for(int k = 0; k < 6; k++){
		int i = add_box(space, cpv(-50.0 + 20.0*k, 10.0), 8.0, 8.0);
		cpBodySetVelocity(bodies[i], cpv(0.0, 90.0 + 8.0*k));
	}
	/* a row of boxes on the ground */
	for(int k = 0; k < 5; k++) add_box(space, cpv(80.0 + 12.0*k, 5.0), 10.0, 10.0);
	/* balls raining on everything, some rolling through the sensor */
	for(int k = 0; k < 10; k++) add_ball(space, cpv(-100.0 + 28.0*k, 80.0 + 9.0*(k % 3)), 3.0 + (k % 3), cpv(15.0 - 3.0*k, 0.0));
	for(int k = 0; k < 3; k++) add_ball(space, cpv(100.0 + 4.0*k, 8.0 + 9.0*k), 3.5, cpv(30.0, 0.0));

	for(int step = 0; step < 240; step++){
		cpSpaceStep(space, 1.0/60.0);
		if(step == 150){
			/* a ball leaves the space while it rests on the ground */
			int victim = -1;
			for(int i = 11; i < nbodies && victim < 0; i++){
				int touching = 0;
				cpBodyEachArbiter(bodies[i], on_ground, &touching);
				if(touching) victim = i;
			}
			printf("order victim %d\n", victim);
			if(victim < 0) continue;
			cpSpaceRemoveShape(space, shapes[victim]);
			cpSpaceRemoveBody(space, bodies[victim]);
			cpShapeFree(shapes[victim]);
			cpBodyFree(bodies[victim]);
			bodies[victim] = NULL; shapes[victim] = NULL;
		}
	}
	printf("order counts %d %d %d %d %d %d %d %d %d %d %d %d %d %ld\n", beginBallGround, sepBallGround, removalSeps,
	       beginBoxBall, refusedBoxBall, sepBoxBall, sensorIn, sensorOut, platformIgnored, platformKept, wildBegins, wildSeps,
	       postCount, defaultContacts);
	printf("sums %a %a %a\n", impulseSum.x, impulseSum.y, keSum);
	for(int i = 0; i < nbodies; i++){
		if(!bodies[i]) continue;
		cpVect p = cpBodyGetPosition(bodies[i]), v = cpBodyGetVelocity(bodies[i]);
		printf("%d %a %a %a %a %a %a\n", i, p.x, p.y, v.x, v.y, cpBodyGetAngle(bodies[i]), cpBodyGetAngularVelocity(bodies[i]));
	}
	for(int i = 0; i < nbodies; i++){
		if(!bodies[i]) continue;
		cpSpaceRemoveShape(space, shapes[i]); cpShapeFree(shapes[i]);
		cpSpaceRemoveBody(space, bodies[i]); cpBodyFree(bodies[i]);
	}
	cpSpaceRemoveShape(space, ground); cpShapeFree(ground);
	cpSpaceRemoveShape(space, platform); cpShapeFree(platform);
	cpSpaceRemoveShape(space, sensor); cpShapeFree(sensor);
	cpSpaceFree(space);
	return 0;
}

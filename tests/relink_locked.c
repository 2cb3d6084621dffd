/*
 * relink_locked.c -- an ordinary Chipmunk2D program (reference public API
 * only) that edits the space from inside a query or an iteration, where
 * the reference refuses it (cpAssertSpaceUnlocked, chipmunk_private.h:273;
 * cpBodySleep's check, cpSpaceComponent.c:318).  argv[1] names the edit:
 * "add" (a body added from a box query), "remove" (a shape removed from
 * cpSpaceEachShape), "type" (a body's type changed from a point query),
 * "sleep" (a body put to sleep from cpSpaceEachBody) or "none" (the same
 * queries with no edit, which must end normally).  It prints whether the
 * space reads as locked inside and after each callback.  Built like
 * relink_program.c.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef RELINK_REFERENCE_HEADERS
#include "chipmunk/chipmunk.h"
#else
#include "chipmunk_gb300.h"
#endif

static cpSpace *space;
static cpBody *ball;
static cpShape *ballShape;
static const char *mode;

static void edit(const char *where)
{
	printf("%s locked %d\n", where, (int)cpSpaceIsLocked(space));
	fflush(stdout);
	if(!strcmp(mode, "add") && !strcmp(where, "box")) cpSpaceAddBody(space, cpBodyNew(1.0, 1.0));
	if(!strcmp(mode, "remove") && !strcmp(where, "each")) cpSpaceRemoveShape(space, ballShape);
	if(!strcmp(mode, "type") && !strcmp(where, "point")) cpBodySetType(ball, CP_BODY_TYPE_KINEMATIC);
	if(!strcmp(mode, "sleep") && !strcmp(where, "bodies")) cpBodySleep(ball);
}

static void box_visit(cpShape *shape, void *data) { (void)shape; (void)data; edit("box"); }
static void each_visit(cpShape *shape, void *data) { (void)shape; (void)data; edit("each"); }
static void body_visit(cpBody *body, void *data) { (void)body; (void)data; edit("bodies"); }
static void point_visit(cpShape *shape, cpVect p, cpFloat d, cpVect g, void *data)
{
	(void)shape; (void)p; (void)d; (void)g; (void)data;
	edit("point");
}

int main(int argc, char **argv)
{
	mode = argc > 1 ? argv[1] : "none";
	space = cpSpaceNew();
	cpSpaceSetGravity(space, cpv(0.0, -100.0));
	cpSpaceSetSleepTimeThreshold(space, 1.0);
	cpShape *ground = cpSpaceAddShape(space, cpSegmentShapeNew(cpSpaceGetStaticBody(space), cpv(-50.0, 0.0), cpv(50.0, 0.0), 0.0));
	ball = cpSpaceAddBody(space, cpBodyNew(1.0, cpMomentForCircle(1.0, 0.0, 5.0, cpvzero)));
	cpBodySetPosition(ball, cpv(0.0, 5.0));
	ballShape = cpSpaceAddShape(space, cpCircleShapeNew(ball, 5.0, cpvzero));
	for(int i = 0; i < 5; i++) cpSpaceStep(space, 1.0/60.0);

	cpSpaceBBQuery(space, cpBBNew(-1.0, -1.0, 1.0, 6.0), CP_SHAPE_FILTER_ALL, box_visit, NULL);
	cpSpacePointQuery(space, cpv(0.0, 4.0), 1.0, CP_SHAPE_FILTER_ALL, point_visit, NULL);
	cpSpaceEachShape(space, each_visit, NULL);
	cpSpaceEachBody(space, body_visit, NULL);
	printf("after locked %d\n", (int)cpSpaceIsLocked(space));

	cpSpaceRemoveShape(space, ballShape); cpShapeFree(ballShape);
	cpSpaceRemoveBody(space, ball); cpBodyFree(ball);
	cpSpaceRemoveShape(space, ground); cpShapeFree(ground);
	cpSpaceFree(space);
	return 0;
}

// Host check of the adjoint building blocks (chipmunk2d_gb300/csrc/cpg_adjoint.cuh)
// against central finite differences:
//  1. one impulse application, the warm start and the pre-step of a contact,
//     against the forward expressions of the device solver;
//  2. the dual-number contact geometry of every pair type, against the
//     device narrow phase itself (cpg_narrow.cuh compiled for the host):
//     values must agree bit for bit, derivatives with central differences.
// Prints one line per group and exits non-zero on a failure.
#define __device__
#define __host__
#define __forceinline__ inline
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#define CUDART_INF INFINITY
#include "cpg_narrow.cuh"
#include "cpg_adjoint.cuh"

static unsigned long long rng_state = 0x9E3779B97F4A7C15ull;
static double urand()
{
	rng_state ^= rng_state << 13; rng_state ^= rng_state >> 7; rng_state ^= rng_state << 17;
	return (double)(rng_state >> 11)*(1.0/9007199254740992.0);
}
static double urange(double a, double b) { return a + (b - a)*urand(); }

static int failures = 0;
static double worst_rel = 0.0;

static void check(const char *what, double adj, double fd, double scale)
{
	double err = fabs(adj - fd)/(fabs(fd) + scale);
	if(err > worst_rel) worst_rel = err;
	if(err > 1e-6){
		if(failures < 20) printf("  FAIL %s: adjoint %.12g finite difference %.12g\n", what, adj, fd);
		failures++;
	}
}

/* ---- 1a. one application, the forward as the device computes it ---- */
struct St { double v[12]; double jN, jT, jB; };   /* A: vx vy w vbx vby wb, B: same */

static void app_forward(const AdjCon &c, St &s, AdjApp *rec)
{
	double *A = s.v, *B = s.v + 6;
	double nx = c.nx, ny = c.ny;
	double vb1x = A[3] + (-c.r1y)*A[5], vb1y = A[4] + c.r1x*A[5];
	double vb2x = B[3] + (-c.r2y)*B[5], vb2y = B[4] + c.r2x*B[5];
	double v1x = A[0] + (-c.r1y)*A[2], v1y = A[1] + c.r1x*A[2];
	double v2x = B[0] + (-c.r2y)*B[2], v2y = B[1] + c.r2x*B[2];
	double vrx = (v2x - v1x) + 0.0, vry = (v2y - v1y) + 0.0;
	double vbx = vb2x - vb1x, vby = vb2y - vb1y;
	if(rec){
		rec->vrx = vrx; rec->vry = vry; rec->vbx = vbx; rec->vby = vby;
		rec->wA = A[2]; rec->wB = B[2]; rec->wbA = A[5]; rec->wbB = B[5];
		rec->jN0 = s.jN; rec->jT0 = s.jT; rec->jB0 = s.jB;
	}
	double vbn = vbx*nx + vby*ny;
	double vrn = vrx*nx + vry*ny;
	double vrt = vrx*(-ny) + vry*nx;
	double jbn = (c.bias - vbn)*c.nMass;
	double jbnOld = s.jB;
	s.jB = dmax(jbnOld + jbn, 0.0);
	double jn = -(c.bounce + vrn)*c.nMass;
	double jnOld = s.jN;
	s.jN = dmax(jnOld + jn, 0.0);
	double jtMax = c.u*s.jN;
	double jt = -vrt*c.tMass;
	double jtOld = s.jT;
	s.jT = dclamp(jtOld + jt, -jtMax, jtMax);
	double db = s.jB - jbnOld;
	double bx = nx*db, by = ny*db;
	A[3] = A[3] + (-bx)*c.minvA; A[4] = A[4] + (-by)*c.minvA; A[5] += c.iinvA*(c.r1x*(-by) - c.r1y*(-bx));
	B[3] = B[3] + bx*c.minvB; B[4] = B[4] + by*c.minvB; B[5] += c.iinvB*(c.r2x*by - c.r2y*bx);
	double djn = s.jN - jnOld, djt = s.jT - jtOld;
	double jx = nx*djn - ny*djt, jy = nx*djt + ny*djn;
	A[0] = A[0] + (-jx)*c.minvA; A[1] = A[1] + (-jy)*c.minvA; A[2] += c.iinvA*(c.r1x*(-jy) - c.r1y*(-jx));
	B[0] = B[0] + jx*c.minvB; B[1] = B[1] + jy*c.minvB; B[2] += c.iinvB*(c.r2x*jy - c.r2y*jx);
	if(rec){ rec->jN1 = s.jN; rec->jT1 = s.jT; rec->jB1 = s.jB; }
}

/* the differentiable inputs: state (15) then constants (13) */
static double *app_param(AdjCon &c, St &s, int i)
{
	if(i < 12) return &s.v[i];
	if(i == 12) return &s.jN;
	if(i == 13) return &s.jT;
	if(i == 14) return &s.jB;
	double *cp[] = { &c.r1x, &c.r1y, &c.r2x, &c.r2y, &c.nx, &c.ny, &c.nMass, &c.tMass, &c.bias, &c.bounce, &c.u, &c.minvA, &c.minvB };
	return cp[i - 15];
}

static double app_loss(const AdjCon &c0, const St &s0, const double *w)
{
	AdjCon c = c0; St s = s0;
	app_forward(c, s, NULL);
	double L = 0.0;
	for(int i = 0; i < 12; i++) L += w[i]*s.v[i];
	return L + w[12]*s.jN + w[13]*s.jT + w[14]*s.jB;
}

static void random_contact(AdjCon &c, St &s, int mode)
{
	double ang = urange(0, 6.283185307179586);
	c.nx = cos(ang); c.ny = sin(ang);
	c.r1x = urange(-2, 2); c.r1y = urange(-2, 2); c.r2x = urange(-2, 2); c.r2y = urange(-2, 2);
	c.minvA = urange(0.2, 2.0); c.minvB = (mode & 1) ? 0.0 : urange(0.2, 2.0);
	c.iinvA = urange(0.1, 1.0); c.iinvB = (mode & 1) ? 0.0 : urange(0.1, 1.0);
	c.nMass = urange(0.2, 1.0); c.tMass = urange(0.2, 1.0);
	c.bias = urange(-1, 3); c.bounce = urange(-2, 1); c.u = urange(0.1, 1.2);
	for(int i = 0; i < 12; i++) s.v[i] = urange(-3, 3);
	s.jN = urange(0, 2); s.jT = urange(-1, 1); s.jB = urange(0, 1);
	if(mode & 2){ s.jN = 0.0; c.bounce = 5.0; }     /* normal clamped at zero */
	if(mode & 4){ c.u = 0.01; }                      /* friction clamped */
}

static void test_application()
{
	int n = 0;
	for(int trial = 0; trial < 4000; trial++){
		AdjCon c; St s;
		random_contact(c, s, trial & 7);
		double w[15];
		for(int i = 0; i < 15; i++) w[i] = urange(-1, 1);
		AdjApp rec;
		{ AdjCon cc = c; St ss = s; app_forward(cc, ss, &rec); }
		AdjBody A = { w[0], w[1], w[2], w[3], w[4], w[5] }, B = { w[6], w[7], w[8], w[9], w[10], w[11] };
		double jNb = w[12], jTb = w[13], jBb = w[14];
		AdjConBar cb; adj_zero(cb);
		app_adjoint(c, rec, A, B, jNb, jTb, jBb, cb);
		double adj[28] = { A.vx, A.vy, A.w, A.vbx, A.vby, A.wb, B.vx, B.vy, B.w, B.vbx, B.vby, B.wb, jNb, jTb, jBb,
			cb.r1x, cb.r1y, cb.r2x, cb.r2y, cb.nx, cb.ny, cb.nMass, cb.tMass, cb.bias, cb.bounce, cb.u, cb.minvA, cb.minvB };
		for(int i = 0; i < 28; i++){
			if((trial & 1) && (i == 6 + 0 || i == 27)) continue;   /* static B: minvB fixed at 0 */
			AdjCon cp = c, cm = c; St sp = s, sm = s;
			double h = 1e-6*(1.0 + fabs(*app_param(cp, sp, i)));
			*app_param(cp, sp, i) += h; *app_param(cm, sm, i) -= h;
			double fd = (app_loss(cp, sp, w) - app_loss(cm, sm, w))/(2*h);
			char name[64]; snprintf(name, sizeof(name), "application trial %d input %d", trial, i);
			check(name, adj[i], fd, 1e-3);
			n++;
		}
	}
	printf("application adjoint: %d checks\n", n);
}

/* ---- 1b. warm start ---- */
static void warm_forward(const AdjCon &c, double jN, double jT, double dtc, double *v)
{
	double nx = c.nx, ny = c.ny;
	double jx = nx*jN - ny*jT, jy = nx*jT + ny*jN;
	jx = jx*dtc; jy = jy*dtc;
	double *A = v, *B = v + 6;
	A[0] = A[0] + (-jx)*c.minvA; A[1] = A[1] + (-jy)*c.minvA; A[2] += c.iinvA*(c.r1x*(-jy) - c.r1y*(-jx));
	B[0] = B[0] + jx*c.minvB; B[1] = B[1] + jy*c.minvB; B[2] += c.iinvB*(c.r2x*jy - c.r2y*jx);
}

static void test_warm()
{
	int n = 0;
	for(int trial = 0; trial < 2000; trial++){
		AdjCon c; St s;
		random_contact(c, s, 0);
		double dtc = urange(0.5, 1.5);
		double w[12];
		for(int i = 0; i < 12; i++) w[i] = (i % 6 < 3) ? urange(-1, 1) : 0.0;
		AdjBody A = { w[0], w[1], w[2], 0, 0, 0 }, B = { w[6], w[7], w[8], 0, 0, 0 };
		double jNb = 0.0, jTb = 0.0;
		AdjConBar cb; adj_zero(cb);
		warm_adjoint(c, s.jN, s.jT, dtc, A, B, jNb, jTb, cb);
		double adj[] = { jNb, jTb, cb.r1x, cb.r1y, cb.r2x, cb.r2y, cb.nx, cb.ny, cb.minvA, cb.minvB };
		for(int i = 0; i < 10; i++){
			double L[2];
			for(int sgn = 0; sgn < 2; sgn++){
				AdjCon cc = c; double jN = s.jN, jT = s.jT;
				double *p[] = { &jN, &jT, &cc.r1x, &cc.r1y, &cc.r2x, &cc.r2y, &cc.nx, &cc.ny, &cc.minvA, &cc.minvB };
				double h = 1e-6*(1.0 + fabs(*p[i]));
				*p[i] += sgn ? -h : h;
				double v[12]; memcpy(v, s.v, sizeof(v));
				warm_forward(cc, jN, jT, dtc, v);
				L[sgn] = 0.0;
				for(int k = 0; k < 12; k++) L[sgn] += w[k]*v[k];
			}
			AdjCon cc = c; double jN = s.jN, jT = s.jT;
			double *p[] = { &jN, &jT, &cc.r1x, &cc.r1y, &cc.r2x, &cc.r2y, &cc.nx, &cc.ny, &cc.minvA, &cc.minvB };
			double h = 1e-6*(1.0 + fabs(*p[i]));
			char name[64]; snprintf(name, sizeof(name), "warm start trial %d input %d", trial, i);
			check(name, adj[i], (L[0] - L[1])/(2*h), 1e-3);
			n++;
		}
	}
	printf("warm-start adjoint: %d checks\n", n);
}

/* ---- 1c. pre-step ---- */
static void test_prestep()
{
	int n = 0;
	for(int trial = 0; trial < 3000; trial++){
		AdjPre p;
		double ang = urange(0, 6.283185307179586);
		p.nx = cos(ang); p.ny = sin(ang);
		p.r1x = urange(-2, 2); p.r1y = urange(-2, 2); p.r2x = urange(-2, 2); p.r2y = urange(-2, 2);
		p.pAx = urange(-5, 5); p.pAy = urange(-5, 5);
		/* put pB so that dist + slop straddles zero across trials */
		double dist = urange(-0.5, 0.4);
		p.pBx = p.pAx; p.pBy = p.pAy;
		double ddx = (p.r2x - p.r1x), ddy = (p.r2y - p.r1y);
		double cur = ddx*p.nx + ddy*p.ny;
		p.pBx += (dist - cur)*p.nx; p.pBy += (dist - cur)*p.ny;
		p.vAx = urange(-3, 3); p.vAy = urange(-3, 3); p.wA = urange(-2, 2);
		p.vBx = urange(-3, 3); p.vBy = urange(-3, 3); p.wB = urange(-2, 2);
		p.minvA = urange(0.2, 2); p.minvB = (trial & 1) ? 0.0 : urange(0.2, 2);
		p.iinvA = urange(0.1, 1); p.iinvB = (trial & 1) ? 0.0 : urange(0.1, 1);
		p.e = urange(0, 0.5); p.biasCoef = 0.2; p.slop = 0.1; p.dt = 1.0/120;
		double w[4] = { urange(-1, 1), urange(-1, 1), urange(-1, 1), urange(-1, 1) };
		AdjPreBar pb; adj_zero(pb);
		prestep_adjoint(p, w[0], w[1], w[2], w[3], pb);
		double adj[] = { pb.r1x, pb.r1y, pb.r2x, pb.r2y, pb.nx, pb.ny, pb.pAx, pb.pAy, pb.pBx, pb.pBy,
			pb.vAx, pb.vAy, pb.wA, pb.vBx, pb.vBy, pb.wB, pb.minvA, pb.minvB, pb.e };
		for(int i = 0; i < 19; i++){
			if((trial & 1) && i == 17) continue;
			double L[2], h = 0;
			for(int sgn = 0; sgn < 2; sgn++){
				AdjPre q = p;
				double *pp[] = { &q.r1x, &q.r1y, &q.r2x, &q.r2y, &q.nx, &q.ny, &q.pAx, &q.pAy, &q.pBx, &q.pBy,
					&q.vAx, &q.vAy, &q.wA, &q.vBx, &q.vBy, &q.wB, &q.minvA, &q.minvB, &q.e };
				h = 1e-7*(1.0 + fabs(*pp[i]));
				*pp[i] += sgn ? -h : h;
				double nm, tm, bi, bo;
				prestep_forward(q, nm, tm, bi, bo);
				L[sgn] = w[0]*nm + w[1]*tm + w[2]*bi + w[3]*bo;
			}
			char name[64]; snprintf(name, sizeof(name), "pre-step trial %d input %d", trial, i);
			check(name, adj[i], (L[0] - L[1])/(2*h), 1e-2);
			n++;
		}
	}
	printf("pre-step adjoint: %d checks\n", n);
}


/* ---- 1d. four lanes per contact against one lane ---- */
static void close_to(const char *what, double a, double b)
{
	/* the lanes add the same terms in another order: rounding only */
	double err = fabs(a - b)/(fabs(b) + 1e-3);
	if(err > 1e-12){
		if(failures < 20) printf("  FAIL %s: lanes %.17g one lane %.17g\n", what, a, b);
		failures++;
	}
}

static void test_quad_lanes()
{
	int n = 0;
	for(int trial = 0; trial < 4000; trial++){
		AdjCon c; St s;
		random_contact(c, s, trial & 7);
		AdjApp rec;
		{ AdjCon cc = c; St ss = s; app_forward(cc, ss, &rec); }
		double w[15];
		for(int i = 0; i < 15; i++) w[i] = urange(-1, 1);
		/* one lane */
		AdjBody A = { w[0], w[1], w[2], w[3], w[4], w[5] }, B = { w[6], w[7], w[8], w[9], w[10], w[11] };
		double jN = w[12], jT = w[13], jB = w[14];
		AdjConBar cb; adj_zero(cb);
		app_adjoint(c, rec, A, B, jN, jT, jB, cb);
		/* four lanes */
		double ax[4], ay[4], aw[4], jbx[4], jby[4];
		AdjLaneBar cl[4];
		for(int q = 0; q < 4; q++){
			int side = q & 1, part = q >> 1;
			const double *o = w + 6*side + 3*part;
			ax[q] = o[0]; ay[q] = o[1]; aw[q] = o[2];
			lane_bar_zero(cl[q]);
			cl[q].jA = part ? w[14] : w[12]; cl[q].j2 = part ? 0.0 : w[13];
			lane_adj_phase1(adj_lane(c, q), adj_lane_rec(rec, side, part), ax[q], ay[q], aw[q], jbx[q], jby[q], cl[q]);
		}
		for(int q = 0; q < 4; q++){
			double Jx = jbx[q] + jbx[q ^ 1], Jy = jby[q] + jby[q ^ 1];
			lane_adj_phase2(adj_lane(c, q), adj_lane_rec(rec, q & 1, q >> 1), Jx, Jy, ax[q], ay[q], aw[q], cl[q]);
		}
		AdjConBar sum;
		lane_bar_sum(cl, sum);
		char nm[64];
		double lanes[] = { ax[0], ay[0], aw[0], ax[2], ay[2], aw[2], ax[1], ay[1], aw[1], ax[3], ay[3], aw[3], cl[0].jA, cl[0].j2, cl[2].jA,
			sum.r1x, sum.r1y, sum.r2x, sum.r2y, sum.nx, sum.ny, sum.nMass, sum.tMass, sum.bias, sum.bounce, sum.u, sum.minvA, sum.minvB };
		double one[] = { A.vx, A.vy, A.w, A.vbx, A.vby, A.wb, B.vx, B.vy, B.w, B.vbx, B.vby, B.wb, jN, jT, jB,
			cb.r1x, cb.r1y, cb.r2x, cb.r2y, cb.nx, cb.ny, cb.nMass, cb.tMass, cb.bias, cb.bounce, cb.u, cb.minvA, cb.minvB };
		for(int i = 0; i < 28; i++){ snprintf(nm, sizeof(nm), "lanes trial %d value %d", trial, i); close_to(nm, lanes[i], one[i]); n++; }
		/* both lanes of a part carry the same accumulator adjoints */
		if(cl[0].jA != cl[1].jA || cl[0].j2 != cl[1].j2 || cl[2].jA != cl[3].jA){ failures++; printf("  FAIL lanes trial %d: pair accumulators differ\n", trial); }
		/* two lanes: lane p takes part p for both bodies */
		{
			double pa[2][3], pb[2][3];
			AdjLaneBar pl[4];
			for(int q = 0; q < 4; q++) lane_bar_zero(pl[q]);
			for(int p = 0; p < 2; p++){
				for(int i = 0; i < 3; i++){ pa[p][i] = w[3*p + i]; pb[p][i] = w[6 + 3*p + i]; }
				pl[2*p].jA = p ? w[14] : w[12]; pl[2*p].j2 = p ? 0.0 : w[13];
				AdjLaneRec ra = adj_lane_rec(rec, 0, p), rb = adj_lane_rec(rec, 1, p);
				pair_adj_apply(adj_lane(c, 2*p), adj_lane(c, 2*p + 1), ra, ra.wown, rb.wown,
					pa[p][0], pa[p][1], pa[p][2], pb[p][0], pb[p][1], pb[p][2], pl[2*p], pl[2*p + 1]);
			}
			AdjConBar ps;
			lane_bar_sum(pl, ps);
			double pairs[] = { pa[0][0], pa[0][1], pa[0][2], pa[1][0], pa[1][1], pa[1][2], pb[0][0], pb[0][1], pb[0][2], pb[1][0], pb[1][1], pb[1][2],
				pl[0].jA, pl[0].j2, pl[2].jA,
				ps.r1x, ps.r1y, ps.r2x, ps.r2y, ps.nx, ps.ny, ps.nMass, ps.tMass, ps.bias, ps.bounce, ps.u, ps.minvA, ps.minvB };
			for(int i = 0; i < 28; i++){ snprintf(nm, sizeof(nm), "pair lanes trial %d value %d", trial, i); close_to(nm, pairs[i], one[i]); n++; }
		}
		/* warm start */
		AdjBody Aw = { w[0], w[1], w[2], 0, 0, 0 }, Bw = { w[6], w[7], w[8], 0, 0, 0 };
		double wN = 0.0, wT = 0.0, dtc = urange(0.5, 1.5);
		AdjConBar wc; adj_zero(wc);
		warm_adjoint(c, s.jN, s.jT, dtc, Aw, Bw, wN, wT, wc);
		double qb[2][2]; AdjLaneBar wl[4];
		for(int q = 0; q < 4; q++) lane_bar_zero(wl[q]);
		for(int q = 0; q < 2; q++){
			const double *o = w + 6*q;
			lane_warm_phase1(adj_lane(c, q), s.jN, s.jT, dtc, o[0], o[1], o[2], qb[q][0], qb[q][1], wl[q]);
		}
		for(int q = 0; q < 2; q++)
			lane_warm_phase2(adj_lane(c, q), s.jN, s.jT, dtc, qb[q][0] + qb[q ^ 1][0], qb[q][1] + qb[q ^ 1][1], wl[q]);
		AdjConBar ws;
		lane_bar_sum(wl, ws);
		double qN[1] = { wl[0].jA }, qT[1] = { wl[0].j2 };
		snprintf(nm, sizeof(nm), "warm lanes trial %d", trial);
		close_to(nm, qN[0], wN); close_to(nm, qT[0], wT);
		close_to(nm, ws.nx, wc.nx); close_to(nm, ws.ny, wc.ny);
		close_to(nm, ws.r1x, wc.r1x); close_to(nm, ws.r2y, wc.r2y);
		close_to(nm, ws.minvA, wc.minvA); close_to(nm, ws.minvB, wc.minvB);
		n += 8;
	}
	printf("four- and two-lane adjoint: %d checks\n", n);
}

/* ---- 2. contact geometry against the narrow phase ---- */
struct LShape {
	int kind;
	double r;
	double c[2];                  /* circle centre (local) */
	double a[2], b[2];            /* segment ends (local) */
	std::vector<double> vx, vy;   /* polygon (local, counter-clockwise) */
};

struct WShape {
	ShapeView view;
	std::vector<double> vx, vy, nx, ny;
	double px, py;
};

static void place(const LShape &l, double px, double py, double ang, unsigned long long hashid, WShape &w)
{
	double cs = cos(ang), sn = sin(ang);
	w.px = px; w.py = py;
	ShapeView &v = w.view;
	memset(&v, 0, sizeof(v));
	v.kind = l.kind; v.r = l.r; v.hashid = hashid;
	v.rot = v2(cs, sn);
	double l_ = INFINITY, b_ = INFINITY, r_ = -INFINITY, t_ = -INFINITY;
	auto tp = [&](double x, double y){ return v2(cs*x - sn*y + px, sn*x + cs*y + py); };
	auto grow = [&](V2 p, double rad){ l_ = fmin(l_, p.x - rad); b_ = fmin(b_, p.y - rad); r_ = fmax(r_, p.x + rad); t_ = fmax(t_, p.y + rad); };
	if(l.kind == CPG_CIRCLE){
		v.p0 = tp(l.c[0], l.c[1]); grow(v.p0, l.r);
	} else if(l.kind == CPG_SEGMENT){
		v.p0 = tp(l.a[0], l.a[1]); v.p1 = tp(l.b[0], l.b[1]);
		double dx = l.b[0] - l.a[0], dy = l.b[1] - l.a[1], len = sqrt(dx*dx + dy*dy);
		double nxl = dy/len, nyl = -dx/len;
		v.n = v2(cs*nxl - sn*nyl, sn*nxl + cs*nyl);
		grow(v.p0, l.r); grow(v.p1, l.r);
	} else {
		int n = (int)l.vx.size();
		w.vx.resize(n); w.vy.resize(n); w.nx.resize(n); w.ny.resize(n);
		for(int i = 0; i < n; i++){
			V2 p = tp(l.vx[i], l.vy[i]);
			w.vx[i] = p.x; w.vy[i] = p.y; grow(p, l.r);
			int j = (i - 1 + n)%n;
			double ex = l.vx[i] - l.vx[j], ey = l.vy[i] - l.vy[j], len = sqrt(ex*ex + ey*ey);
			double nxl = ey/len, nyl = -ex/len;
			w.nx[i] = cs*nxl - sn*nyl; w.ny[i] = sn*nxl + cs*nyl;
		}
		v.count = n;
		v.vx = w.vx.data(); v.vy = w.vy.data(); v.nx = w.nx.data(); v.ny = w.ny.data();
	}
	v.bb = bbnew(l_, b_, r_, t_);
}

static GShape gshape(const WShape &w, int side)
{
	GShape g;
	g.kind = w.view.kind; g.side = side; g.px = w.px; g.py = w.py; g.r = w.view.r;
	g.p0x = w.view.p0.x; g.p0y = w.view.p0.y; g.p1x = w.view.p1.x; g.p1y = w.view.p1.y;
	g.nx = w.view.n.x; g.ny = w.view.n.y;
	g.count = w.view.count;
	g.vx = w.vx.data(); g.vy = w.vy.data(); g.wnx = w.nx.data(); g.wny = w.ny.data();
	return g;
}

static LShape random_shape(int kind)
{
	LShape l; memset(l.c, 0, sizeof(l.c)); l.kind = kind; l.r = 0.0;
	if(kind == CPG_CIRCLE){ l.r = urange(0.5, 2.0); }
	else if(kind == CPG_SEGMENT){
		double len = urange(2, 6);
		l.a[0] = -len/2; l.a[1] = 0; l.b[0] = len/2; l.b[1] = 0; l.r = urange(0, 0.5);
	} else {
		int n = 3 + (int)(urand()*4);
		double base = urange(0, 1), rad = urange(0.8, 2.0);
		for(int i = 0; i < n; i++){
			double a = base + 6.283185307179586*(i + 0.3*urand())/n;
			l.vx.push_back(rad*cos(a)); l.vy.push_back(rad*sin(a));
		}
		if(urand() < 0.3) l.r = urange(0, 0.3);
	}
	return l;
}

static void test_geometry()
{
	int pairs = 0, checks = 0, bitmismatch = 0;
	int kinds[6][2] = { {0, 0}, {0, 1}, {1, 1}, {0, 2}, {1, 2}, {2, 2} };
	for(int trial = 0; trial < 6000; trial++){
		int *k = kinds[trial % 6];
		LShape la = random_shape(k[0]), lb = random_shape(k[1]);
		double pose[6] = { 0, 0, urange(0, 6.28), urange(-2, 2), urange(-2, 2), urange(0, 6.28) };
		WShape wa, wb;
		place(la, pose[0], pose[1], pose[2], 11, wa);
		place(lb, pose[3], pose[4], pose[5], 22, wb);
		NInfo info; int flip;
		collide(wa.view, wb.view, 0u, info, flip);
		if(info.count == 0 || flip) continue;
		pairs++;
		GContacts g;
		geom_contacts(gshape(wa, 0), gshape(wb, 1), info.id, g);
		if(g.count != info.count || g.n.x.v != info.n.x || g.n.y.v != info.n.y){ bitmismatch++; continue; }
		for(int c = 0; c < info.count && c < 2; c++)
			if(g.p1[c].x.v != info.p1[c].x || g.p1[c].y.v != info.p1[c].y || g.p2[c].x.v != info.p2[c].x || g.p2[c].y.v != info.p2[c].y) bitmismatch++;
		for(int j = 0; j < 6; j++){
			double h = 1e-6, out[2][10];
			bool ok = true;
			for(int sgn = 0; sgn < 2; sgn++){
				double q[6]; memcpy(q, pose, sizeof(q));
				q[j] += sgn ? -h : h;
				WShape qa, qb;
				place(la, q[0], q[1], q[2], 11, qa);
				place(lb, q[3], q[4], q[5], 22, qb);
				NInfo qi; int qf;
				collide(qa.view, qb.view, info.id, qi, qf);
				if(qi.count != info.count || qf){ ok = false; break; }
				out[sgn][0] = qi.n.x; out[sgn][1] = qi.n.y;
				for(int c = 0; c < 2; c++){
					out[sgn][2 + 4*c] = qi.p1[c].x; out[sgn][3 + 4*c] = qi.p1[c].y;
					out[sgn][4 + 4*c] = qi.p2[c].x; out[sgn][5 + 4*c] = qi.p2[c].y;
				}
			}
			if(!ok) continue;           /* a feature changed within the step */
			double dual[10] = { g.n.x.d[j], g.n.y.d[j] };
			for(int c = 0; c < 2; c++){
				dual[2 + 4*c] = g.p1[c].x.d[j]; dual[3 + 4*c] = g.p1[c].y.d[j];
				dual[4 + 4*c] = g.p2[c].x.d[j]; dual[5 + 4*c] = g.p2[c].y.d[j];
			}
			for(int o = 0; o < 2 + 4*info.count && o < 10; o++){
				char name[80]; snprintf(name, sizeof(name), "geometry pair %d-%d trial %d pose %d out %d", k[0], k[1], trial, j, o);
				check(name, dual[o], (out[0][o] - out[1][o])/(2*h), 1e-1);
				checks++;
			}
		}
	}
	printf("contact geometry: %d pairs, %d checks, %d value mismatches\n", pairs, checks, bitmismatch);
	if(bitmismatch) failures++;
}

int main()
{
	test_application();
	test_warm();
	test_prestep();
	test_quad_lanes();
	test_geometry();
	printf("worst relative error %.3g, failures %d\n", worst_rel, failures);
	return failures ? 1 : 0;
}

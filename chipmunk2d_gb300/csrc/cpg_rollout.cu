/*
 * cpg_rollout.cu -- recording and reverse pass of the differentiable
 * rollout (reference-order mode, batched worlds).
 *
 * The forward rollout records, per segment of K steps, the solver's inputs
 * (k_tape_*: positions after integration, pre-step velocities, velocities
 * after integration, world geometry, the pre-step rows with their arbiter
 * data, the level structure).  The reverse pass recomputes a segment's
 * solver iterations from them (k_replay_solve, in cpg_kernels.cu), which
 * writes per impulse application the accumulators and velocities the
 * solver saw, then runs the segment's steps in reverse.  A segment that
 * was not recorded is restored from its checkpoint and replayed with the
 * same recording plus the application records.
 *
 * The reverse of one step (cpSpaceStep.c:335-445) runs in the opposite
 * order of the forward (k_adj_solve per world, k_adj_geom per unit,
 * k_adj_accum per world):
 *   1. the adjoints of the impulses stored in the arbiters at the end of
 *      the step seed the contacts' accumulators;
 *   2. the iterations in reverse, levels in reverse (units of one level
 *      touch disjoint dynamic bodies, so they run in parallel without
 *      conflicts), contacts of a unit in reverse, on four or two lanes per
 *      contact (lane_adj_phase1/2, pair_adj_apply);
 *   3. the warm start (lane_warm_phase1/2); the adjoints of the initial
 *      accumulators go to the arbiter contacts they were copied from
 *      (cpArbiterUpdate's hash match);
 *   4. velocity integration (damping) and the bias velocities, which the
 *      step starts at zero;
 *   5. pre-step (prestep_adjoint) and contact geometry (geom_contacts in
 *      dual numbers, geom_adjoint), one thread per unit over all worlds,
 *      then added into the body adjoints level by level;
 *   6. position integration, which turns the pose adjoints into those of
 *      the previous step's velocities and bias velocities.
 * Parameter gradients: 1/m per body (impulses, pre-step masses), and the
 * arbiter's e and u, split onto the two shapes (e = ea*eb, u = ua*ub).
 * External forces are not differentiated (the rollout scenes have none).
 */
#include <cuda_runtime.h>
#include "cpg_device.h"
#include "cpg_adjoint.cuh"

enum { ROW_FIRST_ = 1, ROW_DYN_A_ = 2, ROW_DYN_B_ = 4 };

/* ---- recording ---- */

/* Per-world offsets of this step's rows and level starts in the tape. */
__global__ void k_tape_offsets(cpgSet s)
{
	__shared__ int warpSums[2][32];
	__shared__ int carry[2];
	cpgTape &tp = s.tape;
	int t = tp.step, nw = s.nworlds;
	int *rowOff = tp.rowOff + (size_t)t*(nw + 1);
	int *levOff = tp.levOff + (size_t)t*(nw + 1);
	if(threadIdx.x == 0){ carry[0] = tp.cursor[0]; carry[1] = tp.cursor[1]; }
	__syncthreads();
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
	for(int c0 = 0; c0 < nw; c0 += blockDim.x){
		int w = c0 + threadIdx.x;
		int nr = 0, nl = 0;
		if(w < nw){
			bool active = s.params[w].active != 0;
			const cpgTree &T = s.tree[w];
			nr = active ? T.nunits : 0;
			nl = active ? T.nlevels + 1 : 0;
			tp.params[(size_t)t*nw + w] = s.params[w];
		}
		int xr = nr, xl = nl;
		for(int o = 1; o < 32; o <<= 1){
			int yr = __shfl_up_sync(0xffffffffu, xr, o), yl = __shfl_up_sync(0xffffffffu, xl, o);
			if(lane >= o){ xr += yr; xl += yl; }
		}
		if(lane == 31){ warpSums[0][warp] = xr; warpSums[1][warp] = xl; }
		__syncthreads();
		if(warp == 0){
			int a = (lane < nwarps) ? warpSums[0][lane] : 0, b = (lane < nwarps) ? warpSums[1][lane] : 0;
			for(int o = 1; o < 32; o <<= 1){
				int ya = __shfl_up_sync(0xffffffffu, a, o), yb = __shfl_up_sync(0xffffffffu, b, o);
				if(lane >= o){ a += ya; b += yb; }
			}
			if(lane < nwarps){ warpSums[0][lane] = a; warpSums[1][lane] = b; }
		}
		__syncthreads();
		int pr = (warp > 0) ? warpSums[0][warp - 1] : 0, pl = (warp > 0) ? warpSums[1][warp - 1] : 0;
		if(w < nw){ rowOff[w] = carry[0] + pr + xr - nr; levOff[w] = carry[1] + pl + xl - nl; }
		__syncthreads();
		if(threadIdx.x == 0){ carry[0] += warpSums[0][nwarps - 1]; carry[1] += warpSums[1][nwarps - 1]; }
		__syncthreads();
	}
	if(threadIdx.x == 0){
		rowOff[nw] = carry[0]; levOff[nw] = carry[1];
		tp.cursor[0] = carry[0]; tp.cursor[1] = carry[1];
		if(carry[0] > tp.rowCap || carry[1] > tp.levCap) tp.cursor[2] = 1;
	}
}

__global__ void k_tape_bodies(cpgSet s)
{
	int g = blockIdx.x*blockDim.x + threadIdx.x;
	int nb = s.totalBodies;
	if(g >= nb) return;
	double *b = s.tape.body + (size_t)s.tape.step*8*nb;
	b[g] = s.px[g]; b[nb + g] = s.py[g]; b[2*(size_t)nb + g] = s.ang[g];
	b[3*(size_t)nb + g] = s.vx[g]; b[4*(size_t)nb + g] = s.vy[g]; b[5*(size_t)nb + g] = s.w[g];
	b[6*(size_t)nb + g] = s.ta[g]; b[7*(size_t)nb + g] = s.tb[g];
}

/* The solve's input: velocities after velocity integration. */
__global__ void k_tape_vel(cpgSet s)
{
	int g = blockIdx.x*blockDim.x + threadIdx.x;
	int nb = s.totalBodies;
	if(g >= nb) return;
	double *v = s.tape.vel + (size_t)s.tape.step*3*nb;
	v[g] = s.vx[g]; v[nb + g] = s.vy[g]; v[2*(size_t)nb + g] = s.w[g];
}

__global__ void k_tape_shapes(cpgSet s)
{
	int g = blockIdx.x*blockDim.x + threadIdx.x;
	int ns = s.totalShapes, nv = s.totalVerts;
	if(g < ns){
		double *p = s.tape.shape + (size_t)s.tape.step*6*ns;
		p[g] = s.w0x[g]; p[ns + g] = s.w0y[g]; p[2*(size_t)ns + g] = s.w1x[g];
		p[3*(size_t)ns + g] = s.w1y[g]; p[4*(size_t)ns + g] = s.wnx[g]; p[5*(size_t)ns + g] = s.wny[g];
	}
	if(g < nv){
		double *v = s.tape.verts + (size_t)s.tape.step*4*nv;
		v[g] = s.gvx[g]; v[nv + g] = s.gvy[g]; v[2*(size_t)nv + g] = s.gnx[g]; v[3*(size_t)nv + g] = s.gny[g];
	}
}

__global__ void k_tape_rows(cpgSet s)
{
	int w = blockIdx.y;
	const cpgTape &tp = s.tape;
	int nw = s.nworlds, t = tp.step;
	if(!s.params[w].active) return;
	const cpgWorld &W = s.world[w];
	const cpgTree &T = s.tree[w];
	int ro = tp.rowOff[(size_t)t*(nw + 1) + w], lo = tp.levOff[(size_t)t*(nw + 1) + w];
	int n = T.nunits, nl = T.nlevels + 1;
	const int *start = s.levelStart + W.unitOff + w;
	for(int k = blockIdx.x*blockDim.x + threadIdx.x; k < n; k += gridDim.x*blockDim.x){
		if(ro + k >= tp.rowCap) break;
		const cpgRow &row = s.rows[W.unitOff + k];
		tp.rows[ro + k] = row;
		tp.rowWorld[ro + k] = w;
		int *info = tp.rowInfo + 4*(size_t)(ro + k);
		if(row.kind == 0){
			const cpgArb &arb = s.arbs[row.src];
			info[0] = arb.a; info[1] = arb.b; info[2] = (int)arb.gjk; info[3] = arb.warmSrc;
		} else {
			info[0] = -1; info[1] = -1; info[2] = 0; info[3] = 0;
			atomicOr(&tp.cursor[3], 1);      /* joints are not differentiated */
		}
	}
	for(int l = blockIdx.x*blockDim.x + threadIdx.x; l < nl; l += gridDim.x*blockDim.x)
		if(lo + l < tp.levCap) tp.levels[lo + l] = start[l];
}

static inline int blocks_of(int n, int bs) { return (n + bs - 1)/bs > 0 ? (n + bs - 1)/bs : 1; }

extern "C" int cpg_launch_tape_vel(const cpgSet *s, void *stream)
{
	k_tape_vel<<<blocks_of(s->totalBodies, 256), 256, 0, (cudaStream_t)stream>>>(*s);
	return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

extern "C" int cpg_launch_tape(const cpgSet *s, void *stream)
{
	cudaStream_t st = (cudaStream_t)stream;
	k_tape_offsets<<<1, 1024, 0, st>>>(*s);
	k_tape_bodies<<<blocks_of(s->totalBodies, 256), 256, 0, st>>>(*s);
	int nsv = s->totalShapes > s->totalVerts ? s->totalShapes : s->totalVerts;
	k_tape_shapes<<<blocks_of(nsv, 256), 256, 0, st>>>(*s);
	k_tape_rows<<<dim3(1, s->nworlds), 128, 0, st>>>(*s);
	return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

/* ---- reverse pass ---- */

/* Per contact and lane: the lane's partial sums of the contact's
 * constants' adjoints and the accumulator adjoints its part carries. */
__device__ __forceinline__ AdjLaneBar *lane_scratch(const cpgAdj &a, size_t row, int c, int lane)
{
	return (AdjLaneBar *)(a.con + ((row*2 + (size_t)c)*4 + (size_t)lane)*CPG_ADJ_LANE_DOUBLES);
}

/* The lane's constants of contact c of an arbiter row (g: the lane's body). */
__device__ __forceinline__ AdjLane row_lane(const cpgSet &s, const cpgRow &row, int c, int g, int side, int part)
{
	const cpgRowContact &rc = row.arb.c[c];
	AdjLane L;
	L.side = side; L.part = part;
	L.nx = row.arb.nx; L.ny = row.arb.ny;
	L.minv = s.minv[g]; L.iinv = s.iinv[g];
	L.rx = side ? rc.r2x : rc.r1x; L.ry = side ? rc.r2y : rc.r1y;
	L.c0 = part ? rc.bias : rc.bounce;
	L.nMass = rc.nMass; L.tMass = rc.tMass; L.u = row.arb.u;
	return L;
}

/* A shape's recorded world geometry at step t as a GShape. */
__device__ GShape tape_gshape(const cpgSet &s, int t, int g, int bodyG, int side)
{
	const cpgTape &tp = s.tape;
	int ns = s.totalShapes, nv = s.totalVerts, nb = s.totalBodies;
	const double *sh = tp.shape + (size_t)t*6*ns;
	const double *bd = tp.body + (size_t)t*8*nb;
	GShape r;
	r.kind = s.skind[g];
	r.side = side;
	r.px = bd[bodyG]; r.py = bd[nb + bodyG];
	r.r = s.sr[g];
	r.p0x = sh[g]; r.p0y = sh[ns + g]; r.p1x = sh[2*(size_t)ns + g]; r.p1y = sh[3*(size_t)ns + g];
	r.nx = sh[4*(size_t)ns + g]; r.ny = sh[5*(size_t)ns + g];
	r.count = s.svcount[g];
	int voff = s.world[s.sworld[g]].vertOff + s.svoff[g];
	const double *vt = tp.verts + (size_t)t*4*nv;
	r.vx = vt + voff; r.vy = vt + nv + voff; r.wnx = vt + 2*(size_t)nv + voff; r.wny = vt + 3*(size_t)nv + voff;
	return r;
}

/* Per-unit contributions of the pre-step and geometry adjoints (a.unit). */
enum { U_POSE = 0, U_PA = 6, U_PB = 8, U_VA = 10, U_WA = 12, U_VB = 13, U_WB = 15, U_MA = 16, U_MB = 17, U_E = 18, U_U = 19, U_N = 20 };

/* Steps 1-4 of the reverse step (one block per world, four lanes per
 * unit as in the forward solve): the impulses stored at the end, the
 * iterations and the warm start in reverse, velocity integration.  Worlds
 * of at most `stagedMax` bodies keep their bodies' velocity adjoints (v, w,
 * v_bias, w_bias) in shared memory for the whole solve. */
__global__ void __launch_bounds__(CPG_ADJ_SOLVE_THREADS) k_adj_solve(cpgSet s, cpgAdj a, int t, int stagedMax)
{
	extern __shared__ double sbar[];
	int w = blockIdx.x;
	const cpgTape &tp = s.tape;
	int nw = s.nworlds;
	const cpgParams P = tp.params[(size_t)t*nw + w];
	if(!P.active) return;
	const cpgWorld &W = s.world[w];
	int ro = tp.rowOff[(size_t)t*(nw + 1) + w];
	int n = tp.rowOff[(size_t)t*(nw + 1) + w + 1] - ro;
	int lo = tp.levOff[(size_t)t*(nw + 1) + w];
	int nlev = tp.levOff[(size_t)t*(nw + 1) + w + 1] - lo - 1;
	const int *start = tp.levels + lo;
	const cpgRow *rows = tp.rows + ro;
	const int *info = tp.rowInfo + 4*(size_t)ro;
	int iters = P.iterations;
	int tid = threadIdx.x, nt = blockDim.x;
	int lane4 = tid & 3, quad = tid >> 2, nq = nt >> 2;
	int side = lane4 & 1, part = lane4 >> 1;
	unsigned qmask = 0xFu << (tid & 28);
	unsigned pmask = 0x3u << (tid & 28);     /* the quad's two velocity lanes */
	int nbw = W.nbodies, bo = W.bodyOff;
	/* the contact scratch holds one step's rows */
	int rs = ro - tp.rowOff[(size_t)t*(nw + 1)];
	bool staged = nbw <= stagedMax;
	double *bars = staged ? sbar : a.body + 9*(size_t)bo + 3;
	int bstride = staged ? 6 : 9;
	if(staged)
		for(int i = tid; i < 6*nbw; i += nt) sbar[i] = a.body[9*(size_t)(bo + i/6) + 3 + i%6];

	/* 1. adjoints of the impulses stored at the end of the step */
	for(int k = quad; k < n; k += nq){
		const cpgRow &row = rows[k];
		for(int c = 0; c < 2; c++){
			AdjLaneBar z;
			lane_bar_zero(z);
			if(row.kind == 0 && part == 0 && c < row.count){
				const double *arb = a.arb + 4*(size_t)row.src + 2*c;
				z.jA = arb[0]; z.j2 = arb[1];
			}
			*lane_scratch(a, rs + k, c, lane4) = z;
		}
		__syncwarp(qmask);
		if(lane4 == 0 && row.kind == 0){
			double *arb = a.arb + 4*(size_t)row.src;
			arb[0] = 0.0; arb[1] = 0.0; arb[2] = 0.0; arb[3] = 0.0;
		}
	}
	__syncthreads();

	/* 2. iterations in reverse; a level of more than 8 units runs on two
	 * lanes per contact (one per part, both bodies: ~70 FP64 instructions
	 * per lane for 16 units a warp, against ~59 for 8 on four lanes) */
	bool many = s.nworlds >= 152;
	for(int pass = iters; pass >= 1; pass--){
		for(int l = nlev - 1; l >= 0; l--){
			int U = start[l + 1] - start[l];
			bool two = many ? (((U + 15) >> 4)*70 < ((U + 7) >> 3)*59)
			                : (((2*U + nt - 1)/nt)*70 < ((4*U + nt - 1)/nt)*59);
			if(two){
				int p = tid & 1;
				for(int k = start[l] + (tid >> 1); k < start[l + 1]; k += nt >> 1){
					const cpgRow &row = rows[k];
					if(row.kind != 0) continue;
					bool dynA = (row.flags & ROW_DYN_A_) != 0, dynB = (row.flags & ROW_DYN_B_) != 0;
					double *barA = bars + (size_t)bstride*row.a + 3*p, *barB = bars + (size_t)bstride*row.b + 3*p;
					double ax = 0.0, ay = 0.0, aw = 0.0, bx = 0.0, by = 0.0, bw = 0.0;
					if(dynA){ ax = barA[0]; ay = barA[1]; aw = barA[2]; }
					if(dynB){ bx = barB[0]; by = barB[1]; bw = barB[2]; }
					const AdjApp *rec = (const AdjApp *)tp.app + ((size_t)(ro + k)*iters + (pass - 1))*2;
#pragma unroll
					for(int c = 1; c >= 0; c--){
						if(c >= row.count) continue;
						AdjLane La = row_lane(s, row, c, bo + row.a, 0, p), Lb = row_lane(s, row, c, bo + row.b, 1, p);
						AdjLaneRec t = adj_lane_rec(rec[c], 0, p);
						double wbw = (&rec[c].jN0)[11 + 2*p];
						AdjLaneBar *Sa = lane_scratch(a, rs + k, c, 2*p), *Sb = lane_scratch(a, rs + k, c, 2*p + 1);
						AdjLaneBar Ba = *Sa, Bb = *Sb;
						pair_adj_apply(La, Lb, t, t.wown, wbw, ax, ay, aw, bx, by, bw, Ba, Bb);
						*Sa = Ba; *Sb = Bb;
					}
					if(dynA){ barA[0] = ax; barA[1] = ay; barA[2] = aw; }
					if(dynB){ barB[0] = bx; barB[1] = by; barB[2] = bw; }
				}
				__syncthreads();
				continue;
			}
			for(int k = start[l] + quad; k < start[l + 1]; k += nq){
				const cpgRow &row = rows[k];
				if(row.kind != 0) continue;
				int lb = side ? row.b : row.a;
				bool dyn = (row.flags & (side ? ROW_DYN_B_ : ROW_DYN_A_)) != 0;
				double *bar = bars + (size_t)bstride*lb + 3*part;
				double ax = 0.0, ay = 0.0, aw = 0.0;
				if(dyn){ ax = bar[0]; ay = bar[1]; aw = bar[2]; }
				const AdjApp *rec = (const AdjApp *)tp.app + ((size_t)(ro + k)*iters + (pass - 1))*2;
#pragma unroll
				for(int c = 1; c >= 0; c--){
					if(c >= row.count) continue;
					AdjLane L = row_lane(s, row, c, bo + lb, side, part);
					AdjLaneRec R = adj_lane_rec(rec[c], side, part);
					AdjLaneBar *sc = lane_scratch(a, rs + k, c, lane4);
					AdjLaneBar B = *sc;
					double jbx, jby;
					lane_adj_phase1(L, R, ax, ay, aw, jbx, jby, B);
					jbx += __shfl_xor_sync(qmask, jbx, 1);
					jby += __shfl_xor_sync(qmask, jby, 1);
					lane_adj_phase2(L, R, jbx, jby, ax, ay, aw, B);
					*sc = B;
				}
				if(dyn){ bar[0] = ax; bar[1] = ay; bar[2] = aw; }
			}
			__syncthreads();
		}
	}

	/* 3. warm start on the velocity lanes (the body adjoints pass through),
	 * then the initial accumulators' adjoints go to their source contacts */
	for(int k = quad; k < n; k += nq){
		const cpgRow &row = rows[k];
		if(row.kind != 0) continue;
		if(part == 0 && !(row.flags & ROW_FIRST_)){
			int lb = side ? row.b : row.a;
			bool dyn = (row.flags & (side ? ROW_DYN_B_ : ROW_DYN_A_)) != 0;
			const double *bar = bars + (size_t)bstride*lb;
			double ax = 0.0, ay = 0.0, aw = 0.0;
			if(dyn){ ax = bar[0]; ay = bar[1]; aw = bar[2]; }
			for(int c = row.count - 1; c >= 0; c--){
				AdjLane L = row_lane(s, row, c, bo + lb, side, 0);
				AdjLaneBar *sc = lane_scratch(a, rs + k, c, lane4);
				AdjLaneBar B = *sc;
				double jN = row.arb.c[c].jnAcc, jT = row.arb.c[c].jtAcc;
				double jbx, jby;
				lane_warm_phase1(L, jN, jT, P.dt_coef, ax, ay, aw, jbx, jby, B);
				jbx += __shfl_xor_sync(pmask, jbx, 1);
				jby += __shfl_xor_sync(pmask, jby, 1);
				lane_warm_phase2(L, jN, jT, P.dt_coef, jbx, jby, B);
				*sc = B;
			}
		}
		if(lane4 == 0){
			int src = info[4*k + 3];
			for(int c = 0; c < row.count && c < 2; c++){
				int j = ((src >> (4*c)) & 0xF) - 1;
				if(j >= 0 && j < 2){
					const AdjLaneBar *sc = lane_scratch(a, rs + k, c, 0);
					double *arb = a.arb + 4*(size_t)row.src + 2*j;
					arb[0] += sc->jA; arb[1] += sc->j2;
				}
			}
		}
	}
	__syncthreads();

	/* 4. velocity integration; the bias velocities start the solve at 0 */
	for(int i = tid; i < nbw; i += nt){
		int g = bo + i;
		if(s.btype[g] != CPG_DYNAMIC) continue;
		double *b = a.body + 9*(size_t)g;
		const double *sb = bars + (size_t)bstride*i;
		double vx = sb[0], vy = sb[1], vw = sb[2];
		b[3] = vx*P.damping; b[4] = vy*P.damping; b[5] = vw*P.damping;
		b[6] = 0.0; b[7] = 0.0; b[8] = 0.0;
	}
}

/* Step 5a, one thread per unit of the step (all worlds): the pre-step and
 * contact geometry adjoints of the unit, into a.unit. */
__global__ void k_adj_geom(cpgSet s, cpgAdj a, int t)
{
	const cpgTape &tp = s.tape;
	int nw = s.nworlds;
	int r0 = tp.rowOff[(size_t)t*(nw + 1)], r1 = tp.rowOff[(size_t)t*(nw + 1) + nw];
	int r = r0 + blockIdx.x*blockDim.x + threadIdx.x;
	if(r >= r1) return;
	const cpgRow &row = tp.rows[r];
	double *u = a.unit + (size_t)U_N*(r - r0);
	for(int i = 0; i < U_N; i++) u[i] = 0.0;
	if(row.kind != 0) return;
	int w = tp.rowWorld[r];
	const cpgParams &P = tp.params[(size_t)t*nw + w];
	const cpgWorld &W = s.world[w];
	const int *info = tp.rowInfo + 4*(size_t)r;
	int nb = s.totalBodies;
	const double *bd = tp.body + (size_t)t*8*nb;
	int ga = W.bodyOff + row.a, gb = W.bodyOff + row.b;
	bool da = (row.flags & ROW_DYN_A_) != 0, db = (row.flags & ROW_DYN_B_) != 0;
	double r1bar[4] = {0, 0, 0, 0}, r2bar[4] = {0, 0, 0, 0}, nbx = 0.0, nby = 0.0;
	for(int c = 0; c < row.count && c < 2; c++){
		const cpgRowContact &rc = row.arb.c[c];
		AdjPre p;
		p.r1x = rc.r1x; p.r1y = rc.r1y; p.r2x = rc.r2x; p.r2y = rc.r2y;
		p.nx = row.arb.nx; p.ny = row.arb.ny;
		p.pAx = bd[ga]; p.pAy = bd[nb + ga]; p.pBx = bd[gb]; p.pBy = bd[nb + gb];
		p.vAx = bd[3*(size_t)nb + ga]; p.vAy = bd[4*(size_t)nb + ga]; p.wA = bd[5*(size_t)nb + ga];
		p.vBx = bd[3*(size_t)nb + gb]; p.vBy = bd[4*(size_t)nb + gb]; p.wB = bd[5*(size_t)nb + gb];
		p.minvA = s.minv[ga]; p.minvB = s.minv[gb]; p.iinvA = s.iinv[ga]; p.iinvB = s.iinv[gb];
		p.e = row.arb.e;
		p.biasCoef = P.biasCoef; p.slop = P.slop; p.dt = P.dt;
		/* the four lanes' partial adjoints of the contact's constants */
		AdjLaneBar lb[4];
		for(int q = 0; q < 4; q++) lb[q] = *lane_scratch(a, r - r0, c, q);
		AdjConBar cb;
		lane_bar_sum(lb, cb);
		const AdjConBar *scb = &cb;
		AdjPreBar pb; adj_zero(pb);
		prestep_adjoint(p, scb->nMass, scb->tMass, scb->bias, scb->bounce, pb);
		r1bar[2*c] = scb->r1x + pb.r1x; r1bar[2*c + 1] = scb->r1y + pb.r1y;
		r2bar[2*c] = scb->r2x + pb.r2x; r2bar[2*c + 1] = scb->r2y + pb.r2y;
		nbx += scb->nx + pb.nx; nby += scb->ny + pb.ny;
		u[U_PA] += pb.pAx; u[U_PA + 1] += pb.pAy; u[U_PB] += pb.pBx; u[U_PB + 1] += pb.pBy;
		u[U_VA] += pb.vAx; u[U_VA + 1] += pb.vAy; u[U_WA] += pb.wA;
		u[U_VB] += pb.vBx; u[U_VB + 1] += pb.vBy; u[U_WB] += pb.wB;
		u[U_MA] += scb->minvA + pb.minvA; u[U_MB] += scb->minvB + pb.minvB;
		u[U_E] += pb.e;
		u[U_U] += scb->u;
	}
	/* geometry: the arbiter's shapes in the order the forward stored */
	int sa = W.shapeOff + info[0], sb = W.shapeOff + info[1];
	GShape SA = tape_gshape(s, t, sa, ga, da ? 0 : -1);
	GShape SB = tape_gshape(s, t, sb, gb, db ? 1 : -1);
	GContacts g;
	geom_contacts(SA, SB, (unsigned)info[2], g);
	if(g.count == row.count) geom_adjoint(g, row.count, r1bar, r2bar, nbx, nby, u + U_POSE);
	else atomicOr(&tp.cursor[3], 2);
}

/* Steps 5b and 6 (one block per world): unit contributions into the body
 * adjoints level by level (units of a level touch disjoint dynamic
 * bodies), position integration, per-shape e and u in unit order. */
__global__ void k_adj_accum(cpgSet s, cpgAdj a, int t)
{
	int w = blockIdx.x;
	const cpgTape &tp = s.tape;
	int nw = s.nworlds;
	const cpgParams P = tp.params[(size_t)t*nw + w];
	if(!P.active) return;
	const cpgWorld &W = s.world[w];
	int ro = tp.rowOff[(size_t)t*(nw + 1) + w];
	int n = tp.rowOff[(size_t)t*(nw + 1) + w + 1] - ro;
	int lo = tp.levOff[(size_t)t*(nw + 1) + w];
	int nlev = tp.levOff[(size_t)t*(nw + 1) + w + 1] - lo - 1;
	const int *start = tp.levels + lo;
	const cpgRow *rows = tp.rows + ro;
	const int *info = tp.rowInfo + 4*(size_t)ro;
	int tid = threadIdx.x, nt = blockDim.x;
	int nbw = W.nbodies, bo = W.bodyOff;
	int r0 = tp.rowOff[(size_t)t*(nw + 1)];
	for(int l = 0; l < nlev; l++){
		for(int k = start[l] + tid; k < start[l + 1]; k += nt){
			const cpgRow &row = rows[k];
			if(row.kind != 0) continue;
			const double *u = a.unit + (size_t)U_N*(ro - r0 + k);
			int ga = bo + row.a, gb = bo + row.b;
			if(row.flags & ROW_DYN_A_){
				double *b = a.body + 9*(size_t)ga;
				b[0] += u[U_POSE] + u[U_PA]; b[1] += u[U_POSE + 1] + u[U_PA + 1]; b[2] += u[U_POSE + 2];
				b[3] += u[U_VA]; b[4] += u[U_VA + 1]; b[5] += u[U_WA];
				a.gMinv[ga] += u[U_MA];
			}
			if(row.flags & ROW_DYN_B_){
				double *b = a.body + 9*(size_t)gb;
				b[0] += u[U_POSE + 3] + u[U_PB]; b[1] += u[U_POSE + 4] + u[U_PB + 1]; b[2] += u[U_POSE + 5];
				b[3] += u[U_VB]; b[4] += u[U_VB + 1]; b[5] += u[U_WB];
				a.gMinv[gb] += u[U_MB];
			}
		}
		__syncthreads();
	}
	/* 6. position integration: p' = p + (v + v_bias)*dt, a' = a + (w + w_bias)*dt */
	for(int i = tid; i < nbw; i += nt){
		int g = bo + i;
		if(s.btype[g] != CPG_DYNAMIC) continue;
		double *b = a.body + 9*(size_t)g;
		double dt = P.dt;
		b[3] += b[0]*dt; b[4] += b[1]*dt; b[5] += b[2]*dt;
		b[6] = b[0]*dt; b[7] = b[1]*dt; b[8] = b[2]*dt;
	}
	if(tid == 0){
		for(int k = 0; k < n; k++){
			const cpgRow &row = rows[k];
			if(row.kind != 0) continue;
			int sa = W.shapeOff + info[4*k], sb = W.shapeOff + info[4*k + 1];
			const double *u = a.unit + (size_t)U_N*(ro - r0 + k);
			a.gE[sa] += u[U_E]*s.se[sb]; a.gE[sb] += u[U_E]*s.se[sa];
			a.gU[sa] += u[U_U]*s.su[sb]; a.gU[sb] += u[U_U]*s.su[sa];
		}
	}
}

/* The adjoints of the arbiters' stored impulses follow the arbiters across
 * a checkpoint: slots of arbiters created between checkpoints can differ
 * between the forward and its replay (the table is filled with atomics),
 * so the adjoints are moved by key, from the table `oldKeys` numbering to
 * the current table's. */
__device__ __forceinline__ unsigned long long mix64r(unsigned long long z)
{
	z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
	z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
	return z ^ (z >> 31);
}

__global__ void k_adj_remap(cpgSet s, const unsigned long long *oldKeys, const double *oldArb, double *newArb)
{
	int i = blockIdx.x*blockDim.x + threadIdx.x;
	if(i >= s.arbCap) return;
	double *d = newArb + 4*(size_t)i;
	d[0] = d[1] = d[2] = d[3] = 0.0;
	unsigned long long key = s.keys[i];
	if(key < 2ull) return;
	unsigned mask = (unsigned)s.arbCap - 1;
	unsigned h = (unsigned)mix64r(key) & mask;
	for(int probe = 0; probe < s.arbCap; probe++, h = (h + 1) & mask){
		unsigned long long k = oldKeys[h];
		if(k == key){
			const double *o = oldArb + 4*(size_t)h;
			d[0] = o[0]; d[1] = o[1]; d[2] = o[2]; d[3] = o[3];
			return;
		}
		if(k == 0ull) return;
	}
}

extern "C" int cpg_launch_adjoint_remap(const cpgSet *s, const cpgAdj *a, const void *oldKeys, void *stream)
{
	cudaStream_t st = (cudaStream_t)stream;
	k_adj_remap<<<blocks_of(s->arbCap, 256), 256, 0, st>>>(*s, (const unsigned long long *)oldKeys, a->arb, a->arbTmp);
	cudaMemcpyAsync(a->arb, a->arbTmp, sizeof(double)*4*(size_t)s->arbCap, cudaMemcpyDeviceToDevice, st);
	return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

extern "C" int cpg_launch_adjoint(const cpgSet *s, const cpgAdj *a, int step, int rows, void *stream)
{
	cudaStream_t st = (cudaStream_t)stream;
	/* two warps per world: 16 units of a level per round */
	int stagedMax = s->hostMaxBodies <= CPG_ADJ_STAGED_BODIES ? s->hostMaxBodies : 0;
	k_adj_solve<<<s->nworlds, CPG_ADJ_SOLVE_THREADS, (size_t)stagedMax*6*sizeof(double), st>>>(*s, *a, step, stagedMax);
	k_adj_geom<<<blocks_of(rows, 128), 128, 0, st>>>(*s, *a, step);
	k_adj_accum<<<s->nworlds, 64, 0, st>>>(*s, *a, step);
	return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

/*
 * cpg_kernels.cu -- sm_103a kernels of the cpSpaceStep pipeline and their
 * C-callable launchers.
 *
 * One step of a set of worlds (src/cpSpaceStep.c:335-445) runs as:
 *   k_reset_prev      arbiters solved last step return to NORMAL   (:351-360)
 *   k_integrate_pos   position_func over dynamic bodies             (:364-367)
 *   k_shape_cache     world-space shape data + AABBs                (:371)
 *   k_tree            reference-order broadphase, 1 thread/world    (:372)
 *   k_narrow_classify QueryReject per candidate, buckets by pair kind (:235-244)
 *   k_narrow_collide  cpCollide over the buckets, one kind per warp
 *   k_arb_update      arbiter cache upsert + cpArbiterUpdate        (:246-288)
 *   k_solve_list      order-preserving compaction -> solve list     (:274)
 *   k_arb_filter      age out cached arbiters                       (:380)
 *   k_schedule        exact-order level schedule of the sweep
 *   k_prestep         cpArbiterPreStep + joint preStep              (:383-396)
 *   k_integrate_vel   velocity_func                                 (:399-404)
 *   k_solve           warm start + iterations, level by level       (:406-427)
 *
 * The solver sweep is the reference's serial Gauss-Seidel order.  Two units
 * (arbiters or joints) that share no dynamic body commute exactly, so the
 * schedule assigns every unit the level 1 + max(level of the previous unit
 * touching each of its dynamic bodies); units of one level run in parallel
 * and every body still sees its updates in the reference order, giving
 * bit-identical results.  Static and kinematic bodies have zero inverse
 * mass, are never written, and create no dependency.
 *
 * Compiled with --fmad=false: no multiply-add contraction, so every
 * floating-point operation rounds like the reference's C code.
 */
#include <cstdio>
#include <cuda_runtime.h>
#include <math_constants.h>
#include "cpg_device.h"
#include "cpg_math.cuh"
#include "cpg_tree.cuh"
#include "cpg_narrow.cuh"
#include "cpg_colored.cuh"
#include "cpg_adjoint.cuh"
#include "cpg_mark.cuh"

static long long g_launches = 0;

extern "C" long long cpg_launch_count(int reset)
{
	long long n = g_launches;
	if(reset) g_launches = 0;
	return n;
}

#define LAUNCH(...) do { __VA_ARGS__; g_launches++; } while(0)

/* ------------------------------------------------------------------ */
/* Index maintenance: pending insertions, in add order (cpSpace.c:417-438) */

__device__ TreeCtx make_tree_ctx(const cpgSet *s, int w)
{
	const cpgWorld &W = s->world[w];
	TreeCtx c;
	c.nodes = s->nodes + W.nodeOff;
	c.pairs = s->pairs + W.pairOff;
	c.nodeCap = W.nodeCap;
	c.pairCap = W.pairCap;
	c.T = s->tree + w;
	c.dbins = s->dbins + W.dbinOff;
	c.sbins = s->sbins + W.sbinOff;
	c.dbinCap = W.dbinCap;
	c.sbinCap = W.sbinCap;
	c.bbl = s->bbl + W.shapeOff; c.bbb = s->bbb + W.shapeOff;
	c.bbr = s->bbr + W.shapeOff; c.bbt = s->bbt + W.shapeOff;
	c.sbody = s->sbody + W.shapeOff;
	c.shash = s->shash + W.shapeOff;
	c.vx = s->vx + W.bodyOff; c.vy = s->vy + W.bodyOff;
	c.cands = s->cands + W.candOff;
	c.candCap = W.candCap;
	c.ncand = 0;
	c.collide = 0;
	return c;
}

__global__ void k_apply_ops(cpgSet s)
{
	int w = blockIdx.x*blockDim.x + threadIdx.x;
	if(w >= s.nworlds) return;
	const cpgWorld &W = s.world[w];
	if(W.nops == 0) return;
	TreeCtx c = make_tree_ctx(&s, w);
	for(int i = 0; i < W.nops; i++){
		/* a latched error (a pool ran out mid-insertion) stops the replay,
		 * as it stops the tree step: the tree may hold a half-made leaf */
		if(c.T->error) break;
		cpgOp op = s.ops[W.opOff + i];
		if(s.useHash){
			if(op.kind == CPG_OP_USE_HASH) hash_switch(c, s);
			else hash_apply_op(c, s, op);
			continue;
		}
		if(op.kind == CPG_OP_REMOVE) tree_remove(c, op);
		else if(op.kind == CPG_OP_REINDEX) tree_reindex(c, op);
		else if(op.kind == CPG_OP_REINDEX_STATIC) tree_reindex_static(c);
		else tree_insert(c, op);
	}
}

/* A single space's set rebuilt between steps because objects were added
 * or removed: the tree with its pair cache and leaf sets, and the arbiter
 * cache, carry over into the new set, whose pools are at least as large.
 * Shape indices are the shapes' hash ids, which never change (a removed
 * shape leaves an unused index); body indices are remapped (bodyMap[old]
 * = new, -1 for a body that left).  Arbiters of removed shapes or bodies
 * are dropped, as cpSpaceFilterArbiters drops them (cpSpace.c:481-521).
 * Colours are cleared, so the coloured mode colours afresh. */
__global__ void k_transfer_pools(cpgSet to, cpgSet from)
{
	const cpgWorld &WO = from.world[0], &WN = to.world[0];
	int i0 = blockIdx.x*blockDim.x + threadIdx.x, n = gridDim.x*blockDim.x;
	for(int k = i0; k < WO.nodeCap; k += n) to.nodes[WN.nodeOff + k] = from.nodes[WO.nodeOff + k];
	for(int k = i0; k < WO.pairCap; k += n) to.pairs[WN.pairOff + k] = from.pairs[WO.pairOff + k];
	for(int k = i0; k < WO.dbinCap; k += n) to.dbins[WN.dbinOff + k] = from.dbins[WO.dbinOff + k];
	for(int k = i0; k < WO.sbinCap; k += n) to.sbins[WN.sbinOff + k] = from.sbins[WO.sbinOff + k];
	/* spatial hash grids: the cells and the bin pools carry over (a set
	 * rebuilt from a tree set has fresh grids, made by the switch edit) */
	if(to.useHash && from.useHash && to.numcells == from.numcells){
		for(int k = i0; k < 2*from.numcells; k += n) to.gcells[k] = from.gcells[k];
		for(int w = 0; w < 2; w++){
			for(int k = i0; k < from.gbinCap; k += n){
				to.gbinHandle[(size_t)w*to.gbinCap + k] = from.gbinHandle[(size_t)w*from.gbinCap + k];
				to.gbinNext[(size_t)w*to.gbinCap + k] = from.gbinNext[(size_t)w*from.gbinCap + k];
			}
		}
	}
	if(i0 == 0) to.tree[0] = from.tree[0];
}

__device__ int arb_find_or_insert(const cpgSet &s, unsigned long long key, bool &fresh);

__global__ void k_transfer_arbs(cpgSet to, cpgSet from, const int *bodyMap, const unsigned char *deadShape, int *slotMap)
{
	bool same = (to.arbCap == from.arbCap);
	int oldBodies = from.world[0].nbodies, oldShapes = from.world[0].nshapes;
	for(int k = blockIdx.x*blockDim.x + threadIdx.x; k < from.arbCap; k += gridDim.x*blockDim.x){
		unsigned long long key = from.keys[k];
		slotMap[k] = -1;
		if(key <= CPG_KEY_TOMB){
			if(same) to.keys[k] = key;
			continue;
		}
		cpgArb a = from.arbs[k];
		bool bad = a.ba < 0 || a.ba >= oldBodies || a.bb < 0 || a.bb >= oldBodies ||
			a.a < 0 || a.a >= oldShapes || a.b < 0 || a.b >= oldShapes;
		int ba = bad ? -1 : bodyMap[a.ba], bb = bad ? -1 : bodyMap[a.bb];
		if(ba < 0 || bb < 0 || deadShape[a.a] || deadShape[a.b]){
			if(same) to.keys[k] = CPG_KEY_TOMB;
			continue;
		}
		a.ba = ba; a.bb = bb; a.colorTag = 0;
		int slot = k;
		if(same) to.keys[k] = key;
		else {
			bool fresh;
			slot = arb_find_or_insert(to, key, fresh);
			if(slot < 0){ atomicOr(&to.tree[0].error, CPG_ERR_ARBS); continue; }
		}
		to.arbs[slot] = a;
		slotMap[k] = slot;
	}
}

/* the last solve list (reset by the next step, cpSpaceStep.c:351-360) in
 * its order, without the dropped arbiters */
__global__ void k_transfer_list(cpgSet to, cpgSet from, const int *slotMap)
{
	if(blockIdx.x != 0 || threadIdx.x != 0) return;
	int n = from.tree[0].narb, m = 0;
	for(int i = 0; i < n; i++){
		int slot = slotMap[from.arbList[from.world[0].candOff + i]];
		if(slot >= 0) to.arbList[to.world[0].candOff + m++] = slot;
	}
	to.tree[0].narb = m;
	to.tree[0].ncand = 0;
	to.tree[0].nunits = 0;
}

/* ------------------------------------------------------------------ */

__global__ void k_reset_prev(cpgSet s)
{
	int w = blockIdx.y;
	if(!s.params[w].active) return;
	const cpgWorld &W = s.world[w];
	int n = s.tree[w].narb;
	for(int i = blockIdx.x*blockDim.x + threadIdx.x; i < n; i += gridDim.x*blockDim.x){
		int slot = s.arbList[W.candOff + i];
		s.arbs[slot].state = CPG_ARB_NORMAL;
	}
}

/* cpBody.c:347-357 */
__device__ __forceinline__ void set_transform(const cpgSet &s, int g, double px, double py, double a)
{
	double cx = s.cogx[g], cy = s.cogy[g];
	double rx = cos(a), ry = sin(a);
	s.ta[g] = rx; s.tb[g] = ry;
	s.tc[g] = -ry; s.td[g] = rx;
	s.ttx[g] = px - (cx*rx - cy*ry);
	s.tty[g] = py - (cx*ry + cy*rx);
}

/* cpBody.c:511-522 over each world's dynamic-body list */
__global__ void k_integrate_pos(cpgSet s)
{
	int g = blockIdx.x*blockDim.x + threadIdx.x;
	if(g >= s.totalBodies) return;
	int w = s.bworld[g];
	const cpgParams &P = s.params[w];
	if(!P.active || g - s.world[w].bodyOff >= s.world[w].ndyn) return;
	double dt = P.dt;
	double px = s.px[g] + (s.vx[g] + s.vbx[g])*dt;
	double py = s.py[g] + (s.vy[g] + s.vby[g])*dt;
	double a = s.ang[g] + (s.w[g] + s.wb[g])*dt;
	s.px[g] = px; s.py[g] = py; s.ang[g] = a;
	set_transform(s, g, px, py, a);
	s.vbx[g] = 0.0; s.vby[g] = 0.0; s.wb[g] = 0.0;
}

/* Shape caches: cpShape.c:291-296 (circle), :378-405 (segment),
 * cpPolyShape.c:39-64 (polygon).  Shapes of static bodies are skipped. */
__device__ void cache_shape(const cpgSet &s, int g)
{
	int w = s.sworld[g];
	const cpgWorld &W = s.world[w];
	int body = W.bodyOff + s.sbody[g];
	double ta = s.ta[body], tb = s.tb[body], tc = s.tc[body], td = s.td[body], tx = s.ttx[body], ty = s.tty[body];
	int kind = s.skind[g];
	double r = s.sr[g];
	if(kind == CPG_CIRCLE){
		double cx = s.s0x[g], cy = s.s0y[g];
		double wx = ta*cx + tc*cy + tx, wy = tb*cx + td*cy + ty;
		s.w0x[g] = wx; s.w0y[g] = wy;
		s.bbl[g] = wx - r; s.bbb[g] = wy - r; s.bbr[g] = wx + r; s.bbt[g] = wy + r;
	} else if(kind == CPG_SEGMENT){
		double ax = s.s0x[g], ay = s.s0y[g], bx = s.s1x[g], by = s.s1y[g], nx = s.snx[g], ny = s.sny[g];
		double tax = ta*ax + tc*ay + tx, tay = tb*ax + td*ay + ty;
		double tbx = ta*bx + tc*by + tx, tby = tb*bx + td*by + ty;
		s.w0x[g] = tax; s.w0y[g] = tay; s.w1x[g] = tbx; s.w1y[g] = tby;
		s.wnx[g] = ta*nx + tc*ny; s.wny[g] = tb*nx + td*ny;
		double l, rr, b, t;
		if(tax < tbx){ l = tax; rr = tbx; } else { l = tbx; rr = tax; }
		if(tay < tby){ b = tay; t = tby; } else { b = tby; t = tay; }
		s.bbl[g] = l - r; s.bbb[g] = b - r; s.bbr[g] = rr + r; s.bbt[g] = t + r;
	} else {
		int off = W.vertOff + s.svoff[g];
		int count = s.svcount[g];
		double l = CUDART_INF, rr = -CUDART_INF, b = CUDART_INF, t = -CUDART_INF;
		for(int i = 0; i < count; i++){
			double vx = s.lvx[off + i], vy = s.lvy[off + i];
			double nx = s.lnx[off + i], ny = s.lny[off + i];
			double gx = ta*vx + tc*vy + tx, gy = tb*vx + td*vy + ty;
			s.gvx[off + i] = gx; s.gvy[off + i] = gy;
			s.gnx[off + i] = ta*nx + tc*ny; s.gny[off + i] = tb*nx + td*ny;
			l = dmin(l, gx); rr = dmax(rr, gx);
			b = dmin(b, gy); t = dmax(t, gy);
		}
		s.bbl[g] = l - r; s.bbb[g] = b - r; s.bbr[g] = rr + r; s.bbt[g] = t + r;
	}
}

__global__ void k_shape_cache(cpgSet s)
{
	int g = blockIdx.x*blockDim.x + threadIdx.x;
	if(g >= s.totalShapes) return;
	int w = s.sworld[g];
	if(!s.params[w].active) return;
	int body = s.world[w].bodyOff + s.sbody[g];
	if(s.btype[body] == CPG_STATIC) return;
	cache_shape(s, g);
}

/* cpBBTree.c:638-654: one block per world (largest worlds first); its
 * threads stage the world's node pool in shared memory when it fits and
 * scan the leaves for the ones that moved; thread 0 reinserts those and
 * traverses. */
extern __shared__ cpgNode snodes[];

__global__ void k_tree(cpgSet s, int stagedNodes)
{
	int w = s.worldOrder[blockIdx.x];
	if(!s.params[w].active) return;
	const cpgWorld &W = s.world[w];
	int nn = s.tree[w].nodeTop;
	bool staged = nn <= stagedNodes;
	cpgNode *gnodes = s.nodes + W.nodeOff;
	if(staged){
		for(int i = threadIdx.x; i < nn; i += blockDim.x) snodes[i] = gnodes[i];
		__syncthreads();
	}
	{
		TreeCtx c = make_tree_ctx(&s, w);
		if(staged){ c.nodes = snodes; c.nodeCap = stagedNodes < W.nodeCap ? stagedNodes : W.nodeCap; }
		c.collide = 1;
		tree_reindex_query_block(c, s.parMark != 0);
		if(threadIdx.x == 0) c.T->ncand = c.ncand;
	}
	__syncthreads();
	if(staged){
		nn = s.tree[w].nodeTop;
		for(int i = threadIdx.x; i < nn; i += blockDim.x) gnodes[i] = snodes[i];
	}
}

/* cpSpaceHashReindexQuery for a space on the spatial hash: one thread, in
 * the reference's order (the hash's stamps make each pair's test depend
 * on the handles before it).  When the grids and the handles' fields fit,
 * the block stages them in shared memory first (the walk is a chain of
 * dependent loads) and writes back what the step changed: the dynamic
 * grid and the stamps. */
extern __shared__ int hsmem[];

__global__ void k_hash_step(cpgSet s, int staged)
{
	if(blockIdx.x != 0 || !s.params[0].active) return;
	cpgTree *T = &s.tree[0];
	const cpgWorld &W = s.world[0];
	int nc = s.numcells, cap = s.gbinCap, nn = T->nodeTop;
	cpgNode *gnodes = s.nodes + W.nodeOff;
	int *cells = hsmem, *bh = cells + 2*nc, *bn = bh + 2*cap, *no = bn + 2*cap, *nx = no + nn;
	unsigned *st = (unsigned *)(nx + nn);
	int *rg = (int *)(st + nn);
	if(staged){
		/* the static grid and every handle (the dynamic grid starts empty) */
		int stTop = T->gbinTop[1];
		for(int i = threadIdx.x; i < nc; i += blockDim.x) cells[nc + i] = s.gcells[nc + i];
		for(int i = threadIdx.x; i < stTop; i += blockDim.x){
			bh[cap + i] = s.gbinHandle[cap + i];
			bn[cap + i] = s.gbinNext[cap + i];
		}
		for(int i = threadIdx.x; i < nn; i += blockDim.x){
			int obj = gnodes[i].obj;
			no[i] = obj; nx[i] = gnodes[i].binNext; st[i] = gnodes[i].stamp;
			/* each handle's cell range (cpSpaceHash.c:409-415), exact divisions */
			if(obj >= 0 && obj < W.nshapes){
				int g = W.shapeOff + obj;
				double dim = s.celldim;
				rg[4*i] = floor_int(s.bbl[g]/dim); rg[4*i + 1] = floor_int(s.bbr[g]/dim);
				rg[4*i + 2] = floor_int(s.bbb[g]/dim); rg[4*i + 3] = floor_int(s.bbt[g]/dim);
			} else {
				rg[4*i] = 0; rg[4*i + 1] = -1; rg[4*i + 2] = 0; rg[4*i + 3] = -1;
			}
		}
		__syncthreads();
	}
	if(threadIdx.x == 0){
		TreeCtx c = make_tree_ctx(&s, 0);
		c.collide = 1;
		if(!c.T->error){
			GridCtx g = grid_ctx(s, T, 0), sg = grid_ctx(s, T, 1);
			if(staged){
				g.cells = cells; g.bh = bh; g.bn = bn;
				sg.cells = cells + nc; sg.bh = bh + cap; sg.bn = bn + cap;
				StagedNodes v; v.o = no; v.nx = nx; v.st = st; v.rg = rg;
				hash_reindex_query(c, g, sg, v);
			} else {
				PoolNodes v; v.n = gnodes;
				hash_reindex_query(c, g, sg, v);
			}
		}
		c.T->ncand = c.ncand;
	}
	if(staged){
		__syncthreads();
		int dynTop = T->gbinTop[0];
		for(int i = threadIdx.x; i < nc; i += blockDim.x) s.gcells[i] = cells[i];
		for(int i = threadIdx.x; i < dynTop; i += blockDim.x){
			s.gbinHandle[i] = bh[i];
			s.gbinNext[i] = bn[i];
		}
		for(int i = threadIdx.x; i < nn; i += blockDim.x) gnodes[i].stamp = st[i];
	}
}

/* ---- parallel marking of a single world's tree (cpg_mark.cuh) ----
 * One cooperative launch after k_tree has reinserted the moved leaves with
 * their pairs kept: the marking phases over the leaves (threads take hash
 * bins and walk their chains) and the pair slots, with grid barriers
 * between phases and grid-wide prefix sums.  Candidates, pair lists and
 * slot choice are deterministic. */
#define CPG_MARK_THREADS 256

/* the scratch of cpgSet.markScratch, in the order carve_set sizes it:
 * 9 arrays of nodeCap + 1, 2 of pairCap + 1, incidences, block sums */
__device__ __forceinline__ MarkScratch mark_scratch(const cpgSet &s, const cpgWorld &W, int **freeFlag, int **blockSum)
{
	MarkScratch m;
	int n1 = W.nodeCap + 1, p1 = W.pairCap + 1;
	int *q = s.markScratch;
	m.cnt = q; q += n1;
	m.arrive = q; q += n1;
	m.rank = q; q += n1;
	m.oldB = q; q += n1;
	m.inc = q; q += n1;
	m.incid = q; q += n1;
	m.incCur = q; q += n1;
	m.emit = q; q += n1;
	m.ins = q; q += n1;
	m.freeSlot = q; q += p1;
	*freeFlag = q; q += p1;
	m.incEnt = q; q += 4*(size_t)W.pairCap;
	*blockSum = q;
	m.nFree = 0; m.pairTop = 0; m.incCap = 2*W.pairCap; m.rankCap = n1;
	return m;
}

/* Exclusive scan of a[0, len) by one block: each thread sums a contiguous
 * run, the block scans the run sums, each thread writes its run's
 * prefixes.  Returns the total to every thread. */
__device__ int block_excl_scan(int *a, int len)
{
	__shared__ int wsum[32];
	__shared__ int btot;
	int t = threadIdx.x, lane = t & 31, warp = t >> 5, nw = blockDim.x >> 5;
	int per = (len + (int)blockDim.x - 1)/(int)blockDim.x;
	int i0 = min(len, t*per), i1 = min(len, i0 + per);
	int sum = 0;
	for(int i = i0; i < i1; i++) sum += __ldcg(&a[i]);
	int x = sum;
	for(int o = 1; o < 32; o <<= 1){ int y = __shfl_up_sync(0xffffffffu, x, o); if(lane >= o) x += y; }
	if(lane == 31) wsum[warp] = x;
	__syncthreads();
	if(t == 0){ int acc = 0; for(int k = 0; k < nw; k++){ int v = wsum[k]; wsum[k] = acc; acc += v; } btot = acc; }
	__syncthreads();
	int run = wsum[warp] + x - sum;
	for(int i = i0; i < i1; i++){ int v = __ldcg(&a[i]); a[i] = run; run += v; }
	int tot = btot;
	__syncthreads();
	return tot;
}

/* Exclusive scan of a[0, n) by the whole grid; returns the total. */
__device__ int grid_excl_scan(cg::grid_group &grid, int *a, int n, int *blockSum)
{
	int nb = gridDim.x, b = blockIdx.x;
	int per = (n + nb - 1)/nb;
	int lo = min(n, b*per), hi = min(n, lo + per);
	int tot = block_excl_scan(a + lo, hi - lo);
	if(threadIdx.x == 0) blockSum[b] = tot;
	grid.sync();
	if(b == 0 && threadIdx.x == 0){
		int acc = 0;
		for(int k = 0; k < nb; k++){ int v = __ldcg(&blockSum[k]); blockSum[k] = acc; acc += v; }
		blockSum[nb] = acc;
	}
	grid.sync();
	int base = __ldcg(&blockSum[b]);
	if(base) for(int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) a[i] += base;
	int total = __ldcg(&blockSum[nb]);
	grid.sync();
	return total;
}

/* The phases, in order (each loop over leaves takes hash bins with the
 * same bin-to-thread mapping, so a leaf's own writes are read back by the
 * thread that made them). */
/* A bin chain longer than the node pool is corrupt (a cycle): the walk
 * stops there and latches CPG_ERR_BINS, as the serial re-index scan does. */
__device__ __forceinline__ bool mark_bin_ok(const TreeCtx &c, int n, int g)
{
	if(n < 0) return false;
	if(g > c.nodeCap){ atomicOr(&c.T->error, CPG_ERR_BINS); return false; }
	return true;
}
#define MARK_DYN_LEAVES(n) for(unsigned i_ = gtid; i_ < dsize; i_ += gsz) for(int n = c.dbins[i_], g_ = 0; mark_bin_ok(c, n, g_); n = c.nodes[n].binNext, g_++)
#define MARK_STAT_LEAVES(n) for(unsigned i_ = gtid; i_ < ssize; i_ += gsz) for(int n = c.sbins[i_], g_ = 0; mark_bin_ok(c, n, g_); n = c.nodes[n].binNext, g_++)

__global__ void __launch_bounds__(CPG_MARK_THREADS, 1) k_tree_mark(cpgSet s, int w)
{
	cg::grid_group grid = cg::this_grid();
	const cpgWorld &W = s.world[w];
	TreeCtx c = make_tree_ctx(&s, w);
	c.collide = 1;
	cpgTree *T = c.T;
	if(T->dynRoot < 0 || T->error) return;
	unsigned gtid = blockIdx.x*blockDim.x + threadIdx.x, gsz = gridDim.x*blockDim.x;
	int *freeFlag, *blockSum;
	MarkScratch m = mark_scratch(s, W, &freeFlag, &blockSum);
	int nodeTop = T->nodeTop, pairTop = T->pairTop, nLeaves = (int)T->dynEntries, statRoot = T->statRoot;
	if(nLeaves > m.rankCap || nodeTop > W.nodeCap || pairTop > W.pairCap){
		if(gtid == 0) T->error |= CPG_ERR_NODES;
		return;
	}
	unsigned dsize = T->dynSize, ssize = T->statSize;
	for(int i = gtid; i <= nodeTop; i += gsz){ m.arrive[i] = 0; m.inc[i] = 0; m.incid[i] = 0; m.incCur[i] = 0; }
	grid.sync();
	/* 1: the moved leaves' pairs out of every list */
	MARK_DYN_LEAVES(n) mark_filter_list(c, m, n);
	MARK_STAT_LEAVES(n) mark_filter_list(c, m, n);
	grid.sync();
	/* the pool's free slots; leaf counts bottom up */
	for(int p = gtid; p < pairTop; p += gsz) freeFlag[p] = (__ldcg(&c.pairs[p].pad) == 0) ? 1 : 0;
	MARK_DYN_LEAVES(n) mark_count_up(c, m, n);
	grid.sync();
	/* 2: ranks (the scan's barriers follow) */
	MARK_DYN_LEAVES(n) mark_rank(c, m, n);
	int nFree = grid_excl_scan(grid, freeFlag, pairTop, blockSum);
	for(int p = gtid; p < pairTop; p += gsz) if(__ldcg(&c.pairs[p].pad) == 0) m.freeSlot[__ldcg(&freeFlag[p])] = p;
	/* 3: counts, every moved leaf's before the others' */
	MARK_DYN_LEAVES(n) if(mark_moved(c, n)) mark_count_moved(c, m, n, statRoot);
	grid.sync();
	MARK_DYN_LEAVES(n) if(!mark_moved(c, n)) mark_count_still(c, m, n);
	grid.sync();
	/* 4: offsets */
	int ne = grid_excl_scan(grid, m.emit, nLeaves, blockSum);
	int ni = grid_excl_scan(grid, m.ins, nLeaves, blockSum);
	int nin = grid_excl_scan(grid, m.incid, nodeTop, blockSum);
	m.nFree = nFree; m.pairTop = pairTop;
	int fresh = ni > nFree ? ni - nFree : 0;
	if(ne > c.candCap || pairTop + fresh > c.pairCap || nin > m.incCap){
		if(gtid == 0) T->error |= (ne > c.candCap) ? CPG_ERR_CANDS : CPG_ERR_PAIRS;
		return;
	}
	/* 5: the moved leaves' candidates and new pairs */
	MARK_DYN_LEAVES(n) if(mark_moved(c, n)) mark_write_moved(c, m, n, statRoot);
	grid.sync();
	/* 6, 7: new pairs in front of every list, then the other leaves emit */
	MARK_DYN_LEAVES(n){
		mark_link(c, m, n);
		if(!mark_moved(c, n)) mark_emit_still(c, m, n);
	}
	MARK_STAT_LEAVES(n) mark_link(c, m, n);
	/* the unused free slots back into the pool's list */
	int left = nFree > ni ? nFree - ni : 0;
	for(int k = gtid; k < left; k += gsz){
		int p = __ldcg(&m.freeSlot[ni + k]);
		c.pairs[p].aNext = (k + 1 < left) ? __ldcg(&m.freeSlot[ni + k + 1]) : -1;
	}
	/* every thread is done with mark_moved, which reads the tree's stamp,
	 * before thread 0 advances it */
	grid.sync();
	if(gtid == 0){
		T->freePair = left > 0 ? __ldcg(&m.freeSlot[ni]) : -1;
		T->pairTop = pairTop + fresh;
		T->pairsLive = T->pairTop - left;
		T->ncand = ne;
		T->treeStamp++;
	}
}

/* ------------------------------------------------------------------ */
/* Narrow phase: cpSpaceStep.c:219-244 */

__device__ bool query_reject(const cpgSet &s, const cpgWorld &W, int a, int b)
{
	int ga = W.shapeOff + a, gb = W.shapeOff + b;
	BB ba = bbnew(s.bbl[ga], s.bbb[ga], s.bbr[ga], s.bbt[ga]);
	BB bbb = bbnew(s.bbl[gb], s.bbb[gb], s.bbr[gb], s.bbt[gb]);
	if(!bbintersects(ba, bbb)) return true;
	int bodyA = s.sbody[ga], bodyB = s.sbody[gb];
	if(bodyA == bodyB) return true;
	/* chipmunk_private.h:144-155 */
	unsigned long long groupA = s.sgroup[ga], groupB = s.sgroup[gb];
	if((groupA != 0 && groupA == groupB) || (s.scat[ga] & s.smask[gb]) == 0 || (s.scat[gb] & s.smask[ga]) == 0) return true;
	/* cpSpaceStep.c:204-217: joints with collideBodies off */
	int gBodyA = W.bodyOff + bodyA;
	int start = s.partStart[gBodyA], cnt = s.partCount[gBodyA];
	for(int k = 0; k < cnt; k++) if(s.parts[W.partOff + start + k] == bodyB) return true;
	return false;
}

/* Pair routine of two shape kinds (cpCollision.c:688-726 orders the
 * shapes by kind): 0 circle-circle, 1 circle-segment, 2 segment-segment,
 * 3 circle-poly, 4 segment-poly, 5 poly-poly. */
__device__ __forceinline__ int pair_type(int ka, int kb)
{
	int lo = ka < kb ? ka : kb, hi = ka < kb ? kb : ka;
	int c = lo + hi*3;
	return c == 0 ? 0 : c == 3 ? 1 : c == 4 ? 2 : c == 6 ? 3 : c == 7 ? 4 : 5;
}

/* Pass 1, one thread per candidate: QueryReject; a rejected candidate gets
 * its empty result here, the others are appended to their pair type's
 * bucket (warp-aggregated atomics).  The order inside a bucket is not
 * deterministic and need not be: every candidate's result goes to its own
 * slot. */
__global__ void k_narrow_classify(cpgSet s)
{
	int w = blockIdx.y;
	if(!s.params[w].active) return;
	const cpgWorld &W = s.world[w];
	int n = s.tree[w].ncand;
	int stride = gridDim.x*blockDim.x;
	int lane = threadIdx.x & 31;
	for(int base = blockIdx.x*blockDim.x; base < n; base += stride){
		int i = base + threadIdx.x;
		int t = -1;
		if(i < n){
			cpgCand cd = s.cands[W.candOff + i];
			if(query_reject(s, W, cd.a, cd.b)){
				cpgNarrow out;
				out.count = 0; out.flip = 0; out.idOut = cd.idIn; out.nx = 0.0; out.ny = 0.0;
				s.narrow[W.candOff + i] = out;
				if(cd.pair >= 0) s.pairs[W.pairOff + cd.pair].id = out.idOut;
			} else {
				t = pair_type(s.skind[W.shapeOff + cd.a], s.skind[W.shapeOff + cd.b]);
			}
		}
		unsigned active = __ballot_sync(0xffffffffu, t >= 0);
		if(t >= 0){
			unsigned peers = __match_any_sync(active, t);
			int leader = __ffs(peers) - 1;
			int slot0 = 0;
			if(lane == leader) slot0 = atomicAdd(&s.nbCount[t], __popc(peers));
			slot0 = __shfl_sync(peers, slot0, leader);
			int rank = __popc(peers & ((1u << lane) - 1u));
			s.nbucket[(size_t)t*s.totalCands + slot0 + rank] = W.candOff + i;
		}
	}
}

/* The world whose candidate range holds flat candidate index c. */
__device__ __forceinline__ int world_of_cand(const cpgSet &s, int c)
{
	int lo = 0, hi = s.nworlds - 1;
	while(lo < hi){
		int mid = (lo + hi + 1) >> 1;
		if(s.world[mid].candOff <= c) lo = mid; else hi = mid - 1;
	}
	return lo;
}

/* Pass 2 (cpSpaceStep.c:219-244, cpCollision.c:701-726): the buckets one
 * after another over the whole grid, so that a warp runs one pair routine
 * on 32 candidates that all need it. */
__global__ void __launch_bounds__(128) k_narrow_collide(cpgSet s)
{
	int cnt[CPG_PAIR_TYPES];
	int total = 0;
#pragma unroll
	for(int t = 0; t < CPG_PAIR_TYPES; t++){ cnt[t] = s.nbCount[t]; total += cnt[t]; }
	for(int e = blockIdx.x*blockDim.x + threadIdx.x; e < total; e += gridDim.x*blockDim.x){
		int t = 0, base = 0;
		while(t < CPG_PAIR_TYPES - 1 && e - base >= cnt[t]){ base += cnt[t]; t++; }
		int c = s.nbucket[(size_t)t*s.totalCands + (e - base)];
		int w = world_of_cand(s, c);
		const cpgWorld &W = s.world[w];
		cpgCand cd = s.cands[c];
		NarrowCtx nc; nc.s = &s; nc.shapeBase = W.shapeOff; nc.bodyBase = W.bodyOff; nc.vertBase = W.vertOff;
		ShapeView A = load_shape(nc, cd.a), B = load_shape(nc, cd.b);
		NInfo info;
		int flip;
		collide(A, B, cd.idIn, info, flip);
		cpgNarrow out;
		out.count = info.count > 2 ? 2 : info.count;
		out.flip = flip;
		out.idOut = info.id;
		out.nx = info.n.x; out.ny = info.n.y;
		for(int k = 0; k < out.count; k++){
			out.p1x[k] = info.p1[k].x; out.p1y[k] = info.p1[k].y;
			out.p2x[k] = info.p2[k].x; out.p2y[k] = info.p2[k].y;
			out.hash[k] = info.hash[k];
		}
		s.narrow[c] = out;
		if(cd.pair >= 0) s.pairs[W.pairOff + cd.pair].id = out.idOut;
	}
}

/* ------------------------------------------------------------------ */
/* Arbiter cache (cpSpaceStep.c:246-288, cpArbiter.c:356-414) */

__device__ __forceinline__ unsigned long long arb_key(int w, int a, int b)
{
	unsigned long long lo = (unsigned long long)(a < b ? a : b), hi = (unsigned long long)(a < b ? b : a);
	return (((unsigned long long)w << 42) | (lo << 21) | hi) + 2ull;
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z)
{
	z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
	z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
	return z ^ (z >> 31);
}

/* Returns the slot of `key`, inserting it (fresh arbiter) if absent; -1 when
 * the table is full.  Keys are unique per step, so the only concurrent
 * writers of a slot are inserters of different keys. */
__device__ int arb_find_or_insert(const cpgSet &s, unsigned long long key, bool &fresh)
{
	unsigned mask = (unsigned)s.arbCap - 1;
	unsigned h0 = (unsigned)mix64(key) & mask;
	fresh = false;
	unsigned h = h0;
	for(int probe = 0; probe < s.arbCap; probe++, h = (h + 1) & mask){
		unsigned long long k = *(volatile unsigned long long *)&s.keys[h];
		if(k == key) return (int)h;
		if(k == CPG_KEY_EMPTY) break;
	}
	h = h0;
	for(int probe = 0; probe < s.arbCap; probe++, h = (h + 1) & mask){
		unsigned long long k = *(volatile unsigned long long *)&s.keys[h];
		while(k <= CPG_KEY_TOMB){
			unsigned long long old = atomicCAS(&s.keys[h], k, key);
			if(old == k){ fresh = true; return (int)h; }
			k = old;
		}
	}
	return -1;
}

/* Slot of an arbiter key in the open-addressing table, or -1. */
__device__ int arb_find(const cpgSet &s, unsigned long long key)
{
	unsigned mask = (unsigned)s.arbCap - 1;
	unsigned h = (unsigned)mix64(key) & mask;
	for(int probe = 0; probe < s.arbCap; probe++, h = (h + 1) & mask){
		unsigned long long k = s.keys[h];
		if(k == key) return (int)h;
		if(k == CPG_KEY_EMPTY) break;
	}
	return -1;
}

/* Sleeping edits of a single space, in call order: an arbiter leaves the
 * cache when its body falls asleep (cpSpaceUncacheArbiter,
 * cpSpaceComponent.c:92-101) and rejoins it with the stamp of the call when
 * the body wakes (:50-70).  The arbiter keeps its slot and contacts.  An
 * arbiter whose shape left the space since the edit is gone already. */
__global__ void k_sleep_flags(cpgSet s, const unsigned long long *keys, const int *ops, const unsigned *stamps, int n)
{
	if(blockIdx.x != 0 || threadIdx.x != 0) return;
	for(int i = 0; i < n; i++){
		int slot = arb_find(s, keys[i]);
		if(slot < 0) continue;
		cpgArb &arb = s.arbs[slot];
		if(ops[i]) arb.pad |= CPG_ARB_ASLEEP;
		else { arb.pad &= ~CPG_ARB_ASLEEP; arb.stamp = stamps[i]; }
	}
}

/* The arbiter list of a single space written from its keys, as
 * cpSpaceProcessComponents left it (deletions and appended wakers), and
 * the solver units made from it as k_solve_list makes them.  One block. */
__global__ void k_set_list(cpgSet s, const unsigned long long *keys, int n)
{
	const cpgWorld &W = s.world[0];
	int nunits = n + W.ncons;
	if(n > W.candCap || nunits > W.unitCap){
		if(threadIdx.x == 0){ s.tree[0].error |= CPG_ERR_LEVELS; s.tree[0].narb = 0; s.tree[0].nunits = 0; }
		return;
	}
	for(int i = threadIdx.x; i < n; i += blockDim.x){
		int slot = arb_find(s, keys[i]);
		if(slot < 0){ s.tree[0].error |= CPG_ERR_ARBS; slot = 0; }
		s.arbList[W.candOff + i] = slot;
	}
	__syncthreads();
	if(threadIdx.x == 0){ s.tree[0].narb = n; s.tree[0].nunits = nunits; }
	for(int u = threadIdx.x; u < nunits; u += blockDim.x){
		int a, b;
		if(u < n){
			const cpgArb &arb = s.arbs[s.arbList[W.candOff + u]];
			a = arb.ba; b = arb.bb;
		} else {
			const cpgJoint &j = s.joints[W.consOff + (u - n)];
			a = j.a; b = j.b;
		}
		s.unitA[W.unitOff + u] = (s.btype[W.bodyOff + a] == CPG_DYNAMIC) ? a : -1;
		s.unitB[W.unitOff + u] = (s.btype[W.bodyOff + b] == CPG_DYNAMIC) ? b : -1;
	}
}

__global__ void k_arb_update(cpgSet s)
{
	int w = blockIdx.y;
	const cpgParams &P = s.params[w];
	if(!P.active) return;
	const cpgWorld &W = s.world[w];
	int n = s.tree[w].ncand;
	for(int i = blockIdx.x*blockDim.x + threadIdx.x; i < n; i += gridDim.x*blockDim.x){
		const cpgNarrow nr = s.narrow[W.candOff + i];
		if(nr.count == 0){ s.candArb[W.candOff + i] = -1; continue; }
		cpgCand cd = s.cands[W.candOff + i];
		int ia = nr.flip ? cd.b : cd.a, ib = nr.flip ? cd.a : cd.b;
		bool fresh;
		int slot = arb_find_or_insert(s, arb_key(w, ia, ib), fresh);
		if(slot < 0){ s.tree[w].error |= CPG_ERR_ARBS; s.candArb[W.candOff + i] = -1; continue; }
		cpgArb &arb = s.arbs[slot];
		if(fresh){
			/* cpArbiterInit, cpArbiter.c:260-293 */
			arb.count = 0;
			arb.state = CPG_ARB_FIRST;
			arb.stamp = 0;
			arb.world = w;
			arb.colorTag = 0;     /* no colour yet */
			arb.pad = 0;
			arb.svx = 0.0; arb.svy = 0.0; arb.e = 0.0; arb.u = 0.0;
		}
		int ga = W.shapeOff + ia, gb = W.shapeOff + ib;
		int bodyA = s.sbody[ga], bodyB = s.sbody[gb];
		int gBodyA = W.bodyOff + bodyA, gBodyB = W.bodyOff + bodyB;
		double pax = s.px[gBodyA], pay = s.py[gBodyA], pbx = s.px[gBodyB], pby = s.py[gBodyB];
		cpgContact nc[2];
		int oldCount = arb.count;
		int warmSrc = 0;
		for(int k = 0; k < nr.count; k++){
			cpgContact &con = nc[k];
			con.r1x = nr.p1x[k] - pax; con.r1y = nr.p1y[k] - pay;
			con.r2x = nr.p2x[k] - pbx; con.r2y = nr.p2y[k] - pby;
			con.hash = nr.hash[k];
			con.jnAcc = 0.0; con.jtAcc = 0.0;
			int src = 0;
			for(int j = 0; j < oldCount; j++){
				if(con.hash == arb.c[j].hash){
					con.jnAcc = arb.c[j].jnAcc;
					con.jtAcc = arb.c[j].jtAcc;
					src = j + 1;
				}
			}
			warmSrc |= src << (4*k);
			con.nMass = 0.0; con.tMass = 0.0; con.bounce = 0.0; con.jBias = 0.0; con.bias = 0.0;
		}
		for(int k = 0; k < nr.count; k++) arb.c[k] = nc[k];
		arb.warmSrc = warmSrc;
		arb.gjk = nr.idOut;
		arb.a = ia; arb.b = ib; arb.ba = bodyA; arb.bb = bodyB;
		arb.count = nr.count;
		arb.nx = nr.nx; arb.ny = nr.ny;
		arb.e = s.se[ga]*s.se[gb];
		arb.u = s.su[ga]*s.su[gb];
		double svx = s.svx[gb] - s.svx[ga], svy = s.svy[gb] - s.svy[ga];
		double d = svx*nr.nx + svy*nr.ny;
		arb.svx = svx - nr.nx*d; arb.svy = svy - nr.ny*d;
		if(arb.state == CPG_ARB_CACHED) arb.state = CPG_ARB_FIRST;
		bool sensor = s.ssensor[ga] || s.ssensor[gb];
		bool infinite = (s.m[gBodyA] == CUDART_INF && s.m[gBodyB] == CUDART_INF);
		if(s.bridge){
			/* the record is new this step, or kept (user data) */
			arb.pad = fresh ? (arb.pad | CPG_ARB_FRESH) : (arb.pad & ~CPG_ARB_FRESH);
		}
		if(s.bridge && (s.shost[ga] || s.shost[gb])){
			/* a handler's type: the host runs begin and pre-solve, then
			 * applies the rule below (cpSpaceStep.c:259-283) */
			s.candArb[W.candOff + i] = slot;
		} else if(arb.state != CPG_ARB_IGNORE && !sensor && !infinite){
			s.candArb[W.candOff + i] = slot;
		} else {
			arb.count = 0;
			if(arb.state != CPG_ARB_IGNORE) arb.state = CPG_ARB_NORMAL;
			s.candArb[W.candOff + i] = -1;
		}
		arb.stamp = P.stamp;
	}
}

/* Order-preserving compaction of the pushed arbiters into the solve list,
 * then the solver units (arbiters, then joints) with their dynamic bodies. */
__global__ void k_solve_list(cpgSet s)
{
	int w = blockIdx.x;
	if(!s.params[w].active) return;
	const cpgWorld &W = s.world[w];
	int n = s.tree[w].ncand;
	__shared__ int warpSums[32];
	__shared__ int base;
	if(threadIdx.x == 0) base = 0;
	__syncthreads();
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
	for(int c0 = 0; c0 < n; c0 += blockDim.x){
		int i = c0 + threadIdx.x;
		int slot = (i < n) ? s.candArb[W.candOff + i] : -1;
		bool keep = slot >= 0;
		unsigned ballot = __ballot_sync(0xffffffffu, keep);
		int before = __popc(ballot & ((1u << lane) - 1u));
		if(lane == 0) warpSums[warp] = __popc(ballot);
		__syncthreads();
		int off = 0, total = 0;
		for(int k = 0; k < nwarps; k++){
			if(k < warp) off += warpSums[k];
			total += warpSums[k];
		}
		if(keep) s.arbList[W.candOff + base + off + before] = slot;
		__syncthreads();
		if(threadIdx.x == 0) base += total;
		__syncthreads();
	}
	int narb = base;
	int nunits = narb + W.ncons;
	if(threadIdx.x == 0){
		s.tree[w].narb = narb;
		s.tree[w].nunits = nunits;
		if(nunits > W.unitCap) s.tree[w].error |= CPG_ERR_LEVELS;
	}
	if(nunits > W.unitCap) return;
	for(int u = threadIdx.x; u < nunits; u += blockDim.x){
		int a, b;
		if(u < narb){
			const cpgArb &arb = s.arbs[s.arbList[W.candOff + u]];
			a = arb.ba; b = arb.bb;
		} else {
			const cpgJoint &j = s.joints[W.consOff + (u - narb)];
			a = j.a; b = j.b;
		}
		s.unitA[W.unitOff + u] = (s.btype[W.bodyOff + a] == CPG_DYNAMIC) ? a : -1;
		s.unitB[W.unitOff + u] = (s.btype[W.bodyOff + b] == CPG_DYNAMIC) ? b : -1;
	}
}

/* Coloured mode: the solve list in any order (one colour's units commute),
 * compacted with warp-aggregated atomics, then the joints' units. */
__global__ void k_solve_list_any(cpgSet s, int w)
{
	const cpgWorld &W = s.world[w];
	cpgTree &T = s.tree[w];
	int n = T.ncand;
	int lane = threadIdx.x & 31;
	for(int i0 = blockIdx.x*blockDim.x; i0 < n; i0 += gridDim.x*blockDim.x){
		int i = i0 + threadIdx.x;
		int slot = (i < n) ? s.candArb[W.candOff + i] : -1;
		bool keep = slot >= 0;
		unsigned ballot = __ballot_sync(0xffffffffu, keep);
		int base = 0;
		if(lane == 0 && ballot) base = atomicAdd(&T.narb, __popc(ballot));
		base = __shfl_sync(0xffffffffu, base, 0);
		if(keep){
			int pos = base + __popc(ballot & ((1u << lane) - 1u));
			if(pos < W.unitCap){
				s.arbList[W.candOff + pos] = slot;
				s.unitKey[W.unitOff + pos] = i;
				const cpgArb &arb = s.arbs[slot];
				s.unitA[W.unitOff + pos] = (s.btype[W.bodyOff + arb.ba] == CPG_DYNAMIC) ? arb.ba : -1;
				s.unitB[W.unitOff + pos] = (s.btype[W.bodyOff + arb.bb] == CPG_DYNAMIC) ? arb.bb : -1;
			}
		}
	}
}

__global__ void k_units_joints(cpgSet s, int w)
{
	const cpgWorld &W = s.world[w];
	cpgTree &T = s.tree[w];
	int narb = T.narb, nunits = narb + W.ncons;
	if(blockIdx.x == 0 && threadIdx.x == 0){
		T.nunits = nunits;
		if(nunits > W.unitCap) T.error |= CPG_ERR_LEVELS;
	}
	if(nunits > W.unitCap) return;
	for(int j = blockIdx.x*blockDim.x + threadIdx.x; j < W.ncons; j += gridDim.x*blockDim.x){
		const cpgJoint &jr = s.joints[W.consOff + j];
		s.unitKey[W.unitOff + narb + j] = W.candCap + j;
		s.unitA[W.unitOff + narb + j] = (s.btype[W.bodyOff + jr.a] == CPG_DYNAMIC) ? jr.a : -1;
		s.unitB[W.unitOff + narb + j] = (s.btype[W.bodyOff + jr.b] == CPG_DYNAMIC) ? jr.b : -1;
	}
}

/* cpSpaceStep.c:292-325 */
__global__ void k_arb_filter(cpgSet s)
{
	int i = blockIdx.x*blockDim.x + threadIdx.x;
	if(i >= s.arbCap) return;
	unsigned long long key = s.keys[i];
	if(key <= CPG_KEY_TOMB) return;
	cpgArb &arb = s.arbs[i];
	const cpgParams &P = s.params[arb.world];
	if(!P.active) return;
	/* an arbiter a sleeping body holds is out of the cache (cpSpaceUncacheArbiter) */
	if(arb.pad & CPG_ARB_ASLEEP) return;
	unsigned ticks = P.stamp - arb.stamp;
	/* both bodies static or asleep: the bodies past the world's dynamic
	 * array (sleeping bodies, then static ones) */
	int ndyn = s.world[arb.world].ndyn;
	if(arb.ba >= ndyn && arb.bb >= ndyn) return;
	if(ticks >= 1 && arb.state != CPG_ARB_CACHED){
		arb.state = CPG_ARB_CACHED;
		/* the host calls the separate callbacks */
		if(s.sepSlots){
			int k = atomicAdd(s.sepCount, 1);
			if(k < s.arbCap) s.sepSlots[k] = i;
		}
	}
	if(ticks >= P.persistence){
		arb.count = 0;
		s.keys[i] = CPG_KEY_TOMB;
	} else {
		atomicAdd(&s.stats[3], 1);
	}
}

/* Level schedule of one sweep (arbiters then joints), one thread per
 * world: level(u) = max over u's dynamic bodies of (level of the body's
 * previous unit + 1). */
__global__ void k_schedule(cpgSet s)
{
	int w = blockIdx.x*blockDim.x + threadIdx.x;
	if(w >= s.nworlds || !s.params[w].active) return;
	const cpgWorld &W = s.world[w];
	cpgTree &T = s.tree[w];
	int nunits = T.nunits;
	if(nunits > W.unitCap){ T.nlevels = 0; return; }
	int *last = s.last + W.bodyOff;
	for(int b = 0; b < W.nbodies; b++) last[b] = 0;
	int *lvl = s.unitLevel + W.unitOff;
	const int *ua = s.unitA + W.unitOff, *ub = s.unitB + W.unitOff;
	int nlev = 0;
	for(int u = 0; u < nunits; u++){
		int a = ua[u], b = ub[u];
		int l = 0;
		if(a >= 0 && last[a] > l) l = last[a];
		if(b >= 0 && last[b] > l) l = last[b];
		lvl[u] = l;
		if(a >= 0) last[a] = l + 1;
		if(b >= 0) last[b] = l + 1;
		if(l + 1 > nlev) nlev = l + 1;
	}
	int *start = s.levelStart + W.unitOff + w;
	for(int l = 0; l <= nlev; l++) start[l] = 0;
	for(int u = 0; u < nunits; u++) start[lvl[u] + 1]++;
	for(int l = 0; l < nlev; l++) start[l + 1] += start[l];
	/* stable scatter; start[l] runs as the cursor of level l and is
	 * shifted back afterwards */
	int *order = s.unitOrder + W.unitOff;
	for(int u = 0; u < nunits; u++){
		int l = lvl[u];
		order[start[l]++] = u;
	}
	for(int l = nlev; l > 0; l--) start[l] = start[l - 1];
	start[0] = 0;
	T.nlevels = nlev;
	if(nlev > T.maxChain) T.maxChain = nlev;
}

/* In-place exclusive scan of a[0, len) by one block: each thread sums a
 * contiguous run, warp 0 scans the warps' totals, each thread rewrites its
 * run.  blockDim.x is a multiple of 32, at most 1024. */
__device__ void block_exscan_inplace(int *a, int len)
{
	__shared__ int wsum[32];
	int nt = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	int per = (len + nt - 1)/nt;
	int lo = min(len, tid*per), hi = min(len, lo + per);
	int sum = 0;
	for(int i = lo; i < hi; i++) sum += a[i];
	int x = sum;
	for(int o = 1; o < 32; o <<= 1){
		int y = __shfl_up_sync(0xffffffffu, x, o);
		if(lane >= o) x += y;
	}
	if(lane == 31) wsum[warp] = x;
	__syncthreads();
	if(warp == 0){
		int v = (lane < (nt >> 5)) ? wsum[lane] : 0;
		int z = v;
		for(int o = 1; o < 32; o <<= 1){
			int y = __shfl_up_sync(0xffffffffu, z, o);
			if(lane >= o) z += y;
		}
		wsum[lane] = z - v;
	}
	__syncthreads();
	int run = wsum[warp] + x - sum;
	for(int i = lo; i < hi; i++){ int t = a[i]; a[i] = run; run += t; }
	__syncthreads();
}

/* The level schedule of k_schedule for one large world, by one block of
 * 1024 threads.  The recurrence is a scan in unit order and stays on one
 * thread, but its per-body "last level" array sits in shared memory (a
 * dependent shared load and store per unit instead of two L2 round trips)
 * and the units' body indices are loaded a batch ahead.  The block then
 * counts the units of every level, scans the counts into levelStart and
 * warp 0 scatters the units 32 at a time in unit order (ranks within a
 * warp by __match_any_sync), which is the serial stable scatter's order.
 * Arrays that do not fit in the shared scratch (sh, shInts ints) stay in
 * global memory.  Returns the level count to every thread. */
#define CPG_SCHED_THREADS 1024
#define CPG_SCHED_SMEM_INTS (56*1024)
#define CPG_SCHED_BATCH 16
__device__ int schedule_block(const int *ua, const int *ub, int nunits, int nbodies,
                              int *lastG, int *level, int *levelStart, int *order, int *sh, int shInts)
{
	__shared__ int nlevSh;
	int tid = threadIdx.x, nt = blockDim.x;
	int *last = (nbodies <= shInts) ? sh : lastG;
	for(int b = tid; b < nbodies; b += nt) last[b] = 0;
	__syncthreads();
	if(tid == 0){
		int nlev = 0;
		int na[CPG_SCHED_BATCH], nb[CPG_SCHED_BATCH];
#pragma unroll
		for(int k = 0; k < CPG_SCHED_BATCH; k++){
			na[k] = (k < nunits) ? ua[k] : -1;
			nb[k] = (k < nunits) ? ub[k] : -1;
		}
		for(int u0 = 0; u0 < nunits; u0 += CPG_SCHED_BATCH){
			int ca[CPG_SCHED_BATCH], cb[CPG_SCHED_BATCH];
#pragma unroll
			for(int k = 0; k < CPG_SCHED_BATCH; k++){
				ca[k] = na[k]; cb[k] = nb[k];
				int u = u0 + CPG_SCHED_BATCH + k;
				na[k] = (u < nunits) ? ua[u] : -1;
				nb[k] = (u < nunits) ? ub[u] : -1;
			}
#pragma unroll
			for(int k = 0; k < CPG_SCHED_BATCH; k++){
				int u = u0 + k;
				if(u < nunits){
					int a = ca[k], b = cb[k];
					if(a >= nbodies) a = -1;
					if(b >= nbodies) b = -1;
					int l = 0;
					if(a >= 0 && last[a] > l) l = last[a];
					if(b >= 0 && last[b] > l) l = last[b];
					level[u] = l;
					if(a >= 0) last[a] = l + 1;
					if(b >= 0) last[b] = l + 1;
					if(l + 1 > nlev) nlev = l + 1;
				}
			}
		}
		nlevSh = nlev;
	}
	__syncthreads();
	int nlev = nlevSh;
	/* counts of every level, scanned into the level starts */
	int *cnt = (nlev + 1 <= shInts) ? sh : levelStart;
	for(int l = tid; l <= nlev; l += nt) cnt[l] = 0;
	__syncthreads();
	for(int u = tid; u < nunits; u += nt) atomicAdd(&cnt[level[u]], 1);
	__syncthreads();
	block_exscan_inplace(cnt, nlev + 1);
	if(cnt != levelStart){
		for(int l = tid; l <= nlev; l += nt) levelStart[l] = cnt[l];
	}
	__syncthreads();
	/* stable scatter; cnt[l] runs as level l's cursor */
	if(tid < 32){
		for(int u0 = 0; u0 < nunits; u0 += 32){
			int u = u0 + tid;
			int l = (u < nunits) ? level[u] : -1;
			unsigned peers = __match_any_sync(0xffffffffu, l);
			int rank = __popc(peers & ((1u << tid) - 1u));
			int lead = __ffs(peers) - 1;
			int base = 0;
			if(u < nunits && rank == 0){ base = cnt[l]; cnt[l] = base + __popc(peers); }
			base = __shfl_sync(0xffffffffu, base, lead);
			if(u < nunits) order[base + rank] = u;
			__syncwarp();
		}
	}
	__syncthreads();
	if(cnt == levelStart){
		/* the cursors ended at the next level's start: shift them back */
		if(tid == 0){
			for(int l = nlev; l > 0; l--) levelStart[l] = levelStart[l - 1];
			levelStart[0] = 0;
		}
		__syncthreads();
	}
	return nlev;
}

/* k_schedule for a set of one world (the large single spaces). */
__global__ void __launch_bounds__(CPG_SCHED_THREADS, 1) k_schedule_one(cpgSet s)
{
	extern __shared__ int schedSh[];
	const int w = 0;
	if(!s.params[w].active) return;
	const cpgWorld &W = s.world[w];
	cpgTree &T = s.tree[w];
	int nunits = T.nunits;
	if(nunits > W.unitCap){
		if(threadIdx.x == 0) T.nlevels = 0;
		return;
	}
	int nlev = schedule_block(s.unitA + W.unitOff, s.unitB + W.unitOff, nunits, W.nbodies,
	                          s.last + W.bodyOff, s.unitLevel + W.unitOff, s.levelStart + W.unitOff + w,
	                          s.unitOrder + W.unitOff, schedSh, CPG_SCHED_SMEM_INTS);
	if(threadIdx.x == 0){
		T.nlevels = nlev;
		if(nlev > T.maxChain) T.maxChain = nlev;
	}
}

/* ------------------------------------------------------------------ */
/* Pre-step into solver rows: cpArbiter.c:416-439, cpPivotJoint.c:24-39,
 * cpPinJoint.c:24-46, cpSlideJoint.c:24-56.  Rows are written in schedule
 * order (row k holds unit order[k]). */

#define ROW_FIRST 1
#define ROW_DYN_A 2
#define ROW_DYN_B 4

__device__ __forceinline__ double k_scalar_body(const cpgSet &s, int g, double rx, double ry, double nx, double ny)
{
	double rcn = rx*ny - ry*nx;
	return s.minv[g] + s.iinv[g]*rcn*rcn;
}

/* k_tensor, chipmunk_private.h:228-262: the inverse of the 2x2 effective
 * mass of a point constraint, into the row */
__device__ __forceinline__ void row_k_tensor(const cpgSet &s, int ga, int gb, double r1x, double r1y, double r2x, double r2y, cpgRow &row)
{
	double m_sum = s.minv[ga] + s.minv[gb];
	double k11 = m_sum, k12 = 0.0, k21 = 0.0, k22 = m_sum;
	double ai = s.iinv[ga];
	double r1xsq = r1x*r1x*ai, r1ysq = r1y*r1y*ai, r1nxy = -r1x*r1y*ai;
	k11 += r1ysq; k12 += r1nxy; k21 += r1nxy; k22 += r1xsq;
	double bi = s.iinv[gb];
	double r2xsq = r2x*r2x*bi, r2ysq = r2y*r2y*bi, r2nxy = -r2x*r2y*bi;
	k11 += r2ysq; k12 += r2nxy; k21 += r2nxy; k22 += r2xsq;
	double det = k11*k22 - k12*k21;
	double det_inv = 1.0/det;
	row.jnt.k11 = k22*det_inv; row.jnt.k12 = -k12*det_inv; row.jnt.k21 = -k21*det_inv; row.jnt.k22 = k11*det_inv;
}

/* Pre-steps of the groove, damped spring, damped rotary spring, rotary
 * limit, ratchet, gear and simple motor (cpGrooveJoint.c:24-59,
 * cpDampedSpring.c:29-53, cpDampedRotarySpring.c:29-49,
 * cpRotaryLimitJoint.c:24-46, cpRatchetJoint.c:24-52, cpGearJoint.c:24-35,
 * cpSimpleMotor.c:24-31).  The springs' own impulses are not applied here:
 * they go into the joint record (preJx, preJy) and k_integrate_vel applies
 * them to each body in constraint order, before the velocity update, as
 * the reference's pre-step loop does; the ratchet's angle, a state kept
 * from step to step, is written back to the record. */
__device__ void joint_prestep_more(const cpgSet &s, cpgJoint &jrec, cpgRow &row, int ga, int gb,
                                   double r1x, double r1y, double r2x, double r2y, double biasCoef, double dt)
{
	const cpgJoint &j = jrec;
	double iSum = 0.0;
	switch(j.kind){
	case CPG_GROOVE: {
		double ta_ = s.ta[ga], tb_ = s.tb[ga], tc_ = s.tc[ga], td_ = s.td[ga], tx = s.ttx[ga], ty = s.tty[ga];
		V2 tA = v2(ta_*j.gax + tc_*j.gay + tx, tb_*j.gax + td_*j.gay + ty);
		V2 tB = v2(ta_*j.gbx + tc_*j.gby + tx, tb_*j.gbx + td_*j.gby + ty);
		V2 n = v2(ta_*j.gnx + tc_*j.gny, tb_*j.gnx + td_*j.gny);
		double d = vdot(tA, n);
		V2 pa = v2(s.px[ga], s.py[ga]), pb = v2(s.px[gb], s.py[gb]);
		double tdist = vcross(vadd(pb, v2(r2x, r2y)), n);
		double clamp;
		V2 r1;
		if(tdist <= vcross(tA, n)){ clamp = 1.0; r1 = vsub(tA, pa); }
		else if(tdist >= vcross(tB, n)){ clamp = -1.0; r1 = vsub(tB, pa); }
		else { clamp = 0.0; r1 = vsub(vadd(vmul(vperp(n), -tdist), vmul(n, d)), pa); }
		row.jnt.r1x = r1.x; row.jnt.r1y = r1.y;
		row_k_tensor(s, ga, gb, r1.x, r1.y, r2x, r2y, row);
		V2 delta = vsub(vadd(pb, v2(r2x, r2y)), vadd(pa, r1));
		V2 bias = vclamp(vmul(delta, -biasCoef/dt), j.maxBias);
		row.jnt.biasx = bias.x; row.jnt.biasy = bias.y;
		row.jnt.nx = n.x; row.jnt.ny = n.y;
		row.jnt.clamp = clamp;
		row.jnt.jx = j.jx; row.jnt.jy = j.jy;
		return;
	}
	case CPG_DSPRING: {
		double deltax = (s.px[gb] + r2x) - (s.px[ga] + r1x);
		double deltay = (s.py[gb] + r2y) - (s.py[ga] + r1y);
		double dist = sqrt(deltax*deltax + deltay*deltay);
		double inv = 1.0/(dist ? dist : CUDART_INF);
		double nx = deltax*inv, ny = deltay*inv;
		double k = k_scalar_body(s, ga, r1x, r1y, nx, ny) + k_scalar_body(s, gb, r2x, r2y, nx, ny);
		row.jnt.nx = nx; row.jnt.ny = ny;
		row.jnt.nMass = 1.0/k;
		row.jnt.bias = 0.0;                                  /* target_vrn */
		row.jnt.coef = 1.0 - exp(-j.damping*dt*k);           /* v_coef */
		double j_spring = ((j.restLength - dist)*j.stiffness)*dt;
		row.jnt.jnAcc = j_spring;
		jrec.preJx = nx*j_spring; jrec.preJy = ny*j_spring;
		jrec.r1x = r1x; jrec.r1y = r1y; jrec.r2x = r2x; jrec.r2y = r2y;
		return;
	}
	case CPG_DRSPRING: {
		double moment = s.iinv[ga] + s.iinv[gb];
		row.jnt.nMass = 1.0/moment;                          /* iSum */
		row.jnt.coef = 1.0 - exp(-j.damping*dt*moment);      /* w_coef */
		row.jnt.bias = 0.0;                                  /* target_wrn */
		double j_spring = (((s.ang[ga] - s.ang[gb]) - j.restLength)*j.stiffness)*dt;
		row.jnt.jnAcc = j_spring;
		jrec.preJx = j_spring;
		return;
	}
	case CPG_ROTLIMIT: {
		double dist = s.ang[gb] - s.ang[ga];
		double pdist = 0.0;
		if(dist > j.max) pdist = j.max - dist;
		else if(dist < j.min) pdist = j.min - dist;
		iSum = 1.0/(s.iinv[ga] + s.iinv[gb]);
		row.jnt.nMass = iSum;
		double bias = dclamp(-biasCoef*pdist/dt, -j.maxBias, j.maxBias);
		row.jnt.bias = bias;
		row.jnt.jnAcc = bias ? j.jnAcc : 0.0;
		return;
	}
	case CPG_RATCHET: {
		double angle = j.angle, phase = j.phase, ratchet = j.ratchet;
		double delta = s.ang[gb] - s.ang[ga];
		double diff = angle - delta;
		double pdist = 0.0;
		if(diff*ratchet > 0.0) pdist = diff;
		else jrec.angle = floor((delta - phase)/ratchet)*ratchet + phase;
		iSum = 1.0/(s.iinv[ga] + s.iinv[gb]);
		row.jnt.nMass = iSum;
		double bias = dclamp(-biasCoef*pdist/dt, -j.maxBias, j.maxBias);
		row.jnt.bias = bias;
		row.jnt.jnAcc = bias ? j.jnAcc : 0.0;
		row.jnt.aux1 = ratchet;
		return;
	}
	case CPG_GEAR: {
		iSum = 1.0/(s.iinv[ga]*j.ratioInv + j.ratio*s.iinv[gb]);
		row.jnt.nMass = iSum;
		row.jnt.bias = dclamp(-biasCoef*((s.ang[gb]*j.ratio - s.ang[ga]) - j.phase)/dt, -j.maxBias, j.maxBias);
		row.jnt.jnAcc = j.jnAcc;
		row.jnt.aux1 = j.ratio; row.jnt.aux2 = j.ratioInv;
		return;
	}
	default: /* CPG_MOTOR */
		row.jnt.nMass = 1.0/(s.iinv[ga] + s.iinv[gb]);
		row.jnt.bias = j.rate;
		row.jnt.jnAcc = j.jnAcc;
		return;
	}
}

__global__ void k_build_rows(cpgSet s)
{
	int w = blockIdx.y;
	const cpgParams &P = s.params[w];
	if(!P.active) return;
	const cpgWorld &W = s.world[w];
	const cpgTree &T = s.tree[w];
	int narb = T.narb, nunits = T.nunits;
	if(nunits > W.unitCap) return;
	double dt = P.dt;
	const int *order = s.unitOrder + W.unitOff;
	for(int k = blockIdx.x*blockDim.x + threadIdx.x; k < nunits; k += gridDim.x*blockDim.x){
		int u = order[k];
		cpgRow &row = s.rows[W.unitOff + k];
		if(u < narb){
			int slot = s.arbList[W.candOff + u];
			const cpgArb &arb = s.arbs[slot];
			int ga = W.bodyOff + arb.ba, gb = W.bodyOff + arb.bb;
			row.a = arb.ba; row.b = arb.bb; row.kind = 0; row.count = arb.count; row.src = slot;
			row.flags = (arb.state == CPG_ARB_FIRST ? ROW_FIRST : 0)
				| (s.btype[ga] == CPG_DYNAMIC ? ROW_DYN_A : 0) | (s.btype[gb] == CPG_DYNAMIC ? ROW_DYN_B : 0);
			double nx = arb.nx, ny = arb.ny;
			row.arb.nx = nx; row.arb.ny = ny; row.arb.u = arb.u; row.arb.svx = arb.svx; row.arb.svy = arb.svy;
			row.arb.e = arb.e;        /* for the rollout's pre-step adjoint */
			double dx = s.px[gb] - s.px[ga], dy = s.py[gb] - s.py[ga];
			for(int c = 0; c < arb.count; c++){
				const cpgContact &con = arb.c[c];
				cpgRowContact &rc = row.arb.c[c];
				rc.r1x = con.r1x; rc.r1y = con.r1y; rc.r2x = con.r2x; rc.r2y = con.r2y;
				double kn = k_scalar_body(s, ga, con.r1x, con.r1y, nx, ny) + k_scalar_body(s, gb, con.r2x, con.r2y, nx, ny);
				rc.nMass = 1.0/kn;
				double kt = k_scalar_body(s, ga, con.r1x, con.r1y, -ny, nx) + k_scalar_body(s, gb, con.r2x, con.r2y, -ny, nx);
				rc.tMass = 1.0/kt;
				double ddx = (con.r2x - con.r1x) + dx, ddy = (con.r2y - con.r1y) + dy;
				double dist = ddx*nx + ddy*ny;
				rc.bias = -P.biasCoef*dmin(0.0, dist + P.slop)/dt;
				rc.jBias = 0.0;
				/* relative_velocity, chipmunk_private.h:172-178 */
				double v1x = s.vx[ga] + (-con.r1y)*s.w[ga], v1y = s.vy[ga] + con.r1x*s.w[ga];
				double v2x = s.vx[gb] + (-con.r2y)*s.w[gb], v2y = s.vy[gb] + con.r2x*s.w[gb];
				double vrx = v2x - v1x, vry = v2y - v1y;
				rc.bounce = (vrx*nx + vry*ny)*arb.e;
				rc.jnAcc = con.jnAcc; rc.jtAcc = con.jtAcc;
			}
		} else {
			int jidx = u - narb;
			cpgJoint &jrec = s.joints[W.consOff + jidx];
			const cpgJoint &j = jrec;
			double biasCoef = s.jbias[W.consOff + jidx];
			int ga = W.bodyOff + j.a, gb = W.bodyOff + j.b;
			row.a = j.a; row.b = j.b; row.kind = j.kind; row.count = 0; row.src = jidx;
			row.flags = (s.btype[ga] == CPG_DYNAMIC ? ROW_DYN_A : 0) | (s.btype[gb] == CPG_DYNAMIC ? ROW_DYN_B : 0);
			/* r = transformVect(body, anchor - cog) */
			double lax = j.ax - s.cogx[ga], lay = j.ay - s.cogy[ga];
			double lbx = j.bx - s.cogx[gb], lby = j.by - s.cogy[gb];
			double r1x = s.ta[ga]*lax + s.tc[ga]*lay, r1y = s.tb[ga]*lax + s.td[ga]*lay;
			double r2x = s.ta[gb]*lbx + s.tc[gb]*lby, r2y = s.tb[gb]*lbx + s.td[gb]*lby;
			row.jnt.r1x = r1x; row.jnt.r1y = r1y; row.jnt.r2x = r2x; row.jnt.r2y = r2y;
			row.jnt.maxForce = j.maxForce;
			double deltax = (s.px[gb] + r2x) - (s.px[ga] + r1x);
			double deltay = (s.py[gb] + r2y) - (s.py[ga] + r1y);
			if(j.kind == CPG_PIVOT){
				row_k_tensor(s, ga, gb, r1x, r1y, r2x, r2y, row);
				V2 bias = vclamp(vmul(v2(deltax, deltay), -biasCoef/dt), j.maxBias);
				row.jnt.biasx = bias.x; row.jnt.biasy = bias.y;
				row.jnt.jx = j.jx; row.jnt.jy = j.jy;
			} else if(j.kind == CPG_PIN){
				double dist = sqrt(deltax*deltax + deltay*deltay);
				double inv = 1.0/(dist ? dist : CUDART_INF);
				double nx = deltax*inv, ny = deltay*inv;
				row.jnt.nx = nx; row.jnt.ny = ny;
				double kn = k_scalar_body(s, ga, r1x, r1y, nx, ny) + k_scalar_body(s, gb, r2x, r2y, nx, ny);
				row.jnt.nMass = 1.0/kn;
				row.jnt.bias = dclamp(-biasCoef*(dist - j.dist)/dt, -j.maxBias, j.maxBias);
				row.jnt.jnAcc = j.jnAcc;
			} else if(j.kind == CPG_SLIDE){
				double dist = sqrt(deltax*deltax + deltay*deltay);
				double pdist = 0.0, nx, ny, jn = j.jnAcc;
				if(dist > j.max){
					pdist = dist - j.max;
					V2 n = vnormalize(v2(deltax, deltay));
					nx = n.x; ny = n.y;
				} else if(dist < j.min){
					pdist = j.min - dist;
					V2 n = vneg(vnormalize(v2(deltax, deltay)));
					nx = n.x; ny = n.y;
				} else {
					nx = 0.0; ny = 0.0;
					jn = 0.0;
				}
				row.jnt.nx = nx; row.jnt.ny = ny;
				double kn = k_scalar_body(s, ga, r1x, r1y, nx, ny) + k_scalar_body(s, gb, r2x, r2y, nx, ny);
				row.jnt.nMass = 1.0/kn;
				row.jnt.bias = dclamp(-biasCoef*pdist/dt, -j.maxBias, j.maxBias);
				row.jnt.jnAcc = jn;
			} else {
				joint_prestep_more(s, jrec, row, ga, gb, r1x, r1y, r2x, r2y, biasCoef, dt);
			}
		}
	}
}

/* cpBody.c:493-509, then pack every body's solver state
 * (vx vy w vbx vby wb minv iinv, 64 bytes) */
__device__ void warm_gather(const cpgSet &s, int w, int x, double &vx, double &vy, double &wv, double minv, double iinv);

__global__ void k_integrate_vel(cpgSet s)
{
	int g = blockIdx.x*blockDim.x + threadIdx.x;
	if(g >= s.totalBodies) return;
	int w = s.bworld[g];
	const cpgParams &P = s.params[w];
	if(!P.active) return;
	double vx = s.vx[g], vy = s.vy[g], wv = s.w[g];
	double minv = s.minv[g], iinv = s.iinv[g];
	if(g - s.world[w].bodyOff < s.world[w].ndyn && s.btype[g] != CPG_KINEMATIC){
		double dt = P.dt, damping = P.damping;
		/* the springs' pre-step impulses, in constraint order
		 * (cpDampedSpring.c:51, cpDampedRotarySpring.c:46-47), before the
		 * velocity update that follows the pre-steps (cpSpaceStep.c:395-403) */
		const cpgWorld &W = s.world[w];
		int x = g - W.bodyOff;
		for(int k = 0, n = s.springCount[g]; k < n; k++){
			const cpgJoint &jr = s.joints[W.consOff + s.springs[W.springOff + s.springStart[g] + k]];
			if(jr.kind == CPG_DSPRING){
				if(jr.a == x){
					vx = vx + (-jr.preJx)*minv; vy = vy + (-jr.preJy)*minv;
					wv += iinv*(jr.r1x*(-jr.preJy) - jr.r1y*(-jr.preJx));
				}
				if(jr.b == x){
					vx = vx + jr.preJx*minv; vy = vy + jr.preJy*minv;
					wv += iinv*(jr.r2x*jr.preJy - jr.r2y*jr.preJx);
				}
			} else {
				if(jr.a == x) wv -= jr.preJx*iinv;
				if(jr.b == x) wv += jr.preJx*iinv;
			}
		}
		vx = vx*damping + (P.gx + s.fx[g]*minv)*dt;
		vy = vy*damping + (P.gy + s.fy[g]*minv)*dt;
		wv = wv*damping + s.tq[g]*iinv*dt;
		s.vx[g] = vx; s.vy[g] = vy; s.w[g] = wv;
		s.fx[g] = 0.0; s.fy[g] = 0.0; s.tq[g] = 0.0;
		if(s.warmGather && s.btype[g] == CPG_DYNAMIC && s.colorCursor[13] == 0)
			warm_gather(s, w, g - s.world[w].bodyOff, vx, vy, wv, minv, iinv);
	}
	double2 *pb = (double2 *)(s.pbody + 8*(size_t)g);
	pb[0] = make_double2(vx, vy);
	pb[1] = make_double2(wv, s.vbx[g]);
	pb[2] = make_double2(s.vby[g], s.wb[g]);
	pb[3] = make_double2(minv, iinv);
}

/* ------------------------------------------------------------------ */
/* Solver units on rows: cpArbiter.c:441-498, joint applyCachedImpulse /
 * applyImpulse.  Bodies come from the packed state; only dynamic bodies
 * are written back (the others have zero inverse mass, so the reference's
 * update leaves them unchanged). */

struct BodyRef { double vx, vy, w, vbx, vby, wb, minv, iinv; };

template<bool CG>
__device__ __forceinline__ BodyRef load_pbody(const double *base, int b)
{
	const double2 *p = (const double2 *)(base + 8*(size_t)b);
	double2 x0, x1, x2, x3;
	if(CG){ x0 = __ldcg(p); x1 = __ldcg(p + 1); x2 = __ldcg(p + 2); x3 = __ldcg(p + 3); }
	else { x0 = p[0]; x1 = p[1]; x2 = p[2]; x3 = p[3]; }
	BodyRef r;
	r.vx = x0.x; r.vy = x0.y; r.w = x1.x; r.vbx = x1.y; r.vby = x2.x; r.wb = x2.y; r.minv = x3.x; r.iinv = x3.y;
	return r;
}

__device__ __forceinline__ void store_pbody(double *base, int b, const BodyRef &r)
{
	double2 *p = (double2 *)(base + 8*(size_t)b);
	p[0] = make_double2(r.vx, r.vy);
	p[1] = make_double2(r.w, r.vbx);
	p[2] = make_double2(r.vby, r.wb);
}

/* chipmunk_private.h:193-210 */
__device__ __forceinline__ void apply_impulse(BodyRef &b, double jx, double jy, double rx, double ry)
{
	b.vx = b.vx + jx*b.minv;
	b.vy = b.vy + jy*b.minv;
	b.w += b.iinv*(rx*jy - ry*jx);
}

__device__ __forceinline__ void apply_impulses(BodyRef &a, BodyRef &b, double r1x, double r1y, double r2x, double r2y, double jx, double jy)
{
	apply_impulse(a, -jx, -jy, r1x, r1y);
	apply_impulse(b, jx, jy, r2x, r2y);
}

__device__ __forceinline__ void apply_bias_impulse(BodyRef &b, double jx, double jy, double rx, double ry)
{
	b.vbx = b.vbx + jx*b.minv;
	b.vby = b.vby + jy*b.minv;
	b.wb += b.iinv*(rx*jy - ry*jx);
}

/* warm start: cpArbiter.c:441-455, joint applyCachedImpulse */
__device__ __forceinline__ void row_apply_cached(const cpgRow &row, BodyRef &A, BodyRef &B, double dt_coef)
{
	if(row.kind == 0){
		if(row.flags & ROW_FIRST) return;
		double nx = row.arb.nx, ny = row.arb.ny;
#pragma unroll
		for(int k = 0; k < 2; k++){
			if(k >= row.count) break;
			const cpgRowContact &con = row.arb.c[k];
			/* j = rotate(n, (jnAcc, jtAcc)) * dt_coef */
			double jx = nx*con.jnAcc - ny*con.jtAcc, jy = nx*con.jtAcc + ny*con.jnAcc;
			apply_impulses(A, B, con.r1x, con.r1y, con.r2x, con.r2y, jx*dt_coef, jy*dt_coef);
		}
	} else if(row.kind == CPG_PIVOT || row.kind == CPG_GROOVE){
		apply_impulses(A, B, row.jnt.r1x, row.jnt.r1y, row.jnt.r2x, row.jnt.r2y, row.jnt.jx*dt_coef, row.jnt.jy*dt_coef);
	} else if(row.kind == CPG_PIN || row.kind == CPG_SLIDE){
		double s_ = row.jnt.jnAcc*dt_coef;
		apply_impulses(A, B, row.jnt.r1x, row.jnt.r1y, row.jnt.r2x, row.jnt.r2y, row.jnt.nx*s_, row.jnt.ny*s_);
	} else if(row.kind == CPG_ROTLIMIT || row.kind == CPG_RATCHET || row.kind == CPG_MOTOR || row.kind == CPG_GEAR){
		/* cpRotaryLimitJoint.c:48-57, cpRatchetJoint.c:54-62, cpGearJoint.c:37-46, cpSimpleMotor.c:33-41 */
		double j = row.jnt.jnAcc*dt_coef;
		A.w -= (row.kind == CPG_GEAR) ? j*A.iinv*row.jnt.aux2 : j*A.iinv;
		B.w += j*B.iinv;
	}
	/* the springs keep no cached impulse (cpDampedSpring.c:55, cpDampedRotarySpring.c:51) */
}

/* One iteration of the groove, springs and rotary joints:
 * cpGrooveJoint.c:61-94, cpDampedSpring.c:57-77, cpDampedRotarySpring.c:53-72,
 * cpRotaryLimitJoint.c:59-85, cpRatchetJoint.c:64-87, cpGearJoint.c:48-67,
 * cpSimpleMotor.c:43-61 */
__device__ __noinline__ void row_apply_more(cpgRow &row, BodyRef &A, BodyRef &B, double dt)
{
	switch(row.kind){
	case CPG_GROOVE: {
		double v1x = A.vx + (-row.jnt.r1y)*A.w, v1y = A.vy + row.jnt.r1x*A.w;
		double v2x = B.vx + (-row.jnt.r2y)*B.w, v2y = B.vy + row.jnt.r2x*B.w;
		double vrx = v2x - v1x, vry = v2y - v1y;
		double ex = row.jnt.biasx - vrx, ey = row.jnt.biasy - vry;
		double jx = ex*row.jnt.k11 + ey*row.jnt.k12, jy = ex*row.jnt.k21 + ey*row.jnt.k22;
		double oldx = row.jnt.jx, oldy = row.jnt.jy;
		V2 acc = v2(oldx + jx, oldy + jy);
		V2 n = v2(row.jnt.nx, row.jnt.ny);
		/* grooveConstrain: inside the groove's ends only the normal part, at
		 * an end also the part pushing back in */
		V2 jc = (row.jnt.clamp*vcross(acc, n) > 0.0) ? acc : vmul(n, vdot(acc, n)/vdot(n, n));
		acc = vclamp(jc, row.jnt.maxForce*dt);
		row.jnt.jx = acc.x; row.jnt.jy = acc.y;
		apply_impulses(A, B, row.jnt.r1x, row.jnt.r1y, row.jnt.r2x, row.jnt.r2y, acc.x - oldx, acc.y - oldy);
		return;
	}
	case CPG_DSPRING: {
		double v1x = A.vx + (-row.jnt.r1y)*A.w, v1y = A.vy + row.jnt.r1x*A.w;
		double v2x = B.vx + (-row.jnt.r2y)*B.w, v2y = B.vy + row.jnt.r2x*B.w;
		double vrn = (v2x - v1x)*row.jnt.nx + (v2y - v1y)*row.jnt.ny;
		double v_damp = (row.jnt.bias - vrn)*row.jnt.coef;
		row.jnt.bias = vrn + v_damp;
		double j_damp = v_damp*row.jnt.nMass;
		row.jnt.jnAcc += j_damp;
		apply_impulses(A, B, row.jnt.r1x, row.jnt.r1y, row.jnt.r2x, row.jnt.r2y, row.jnt.nx*j_damp, row.jnt.ny*j_damp);
		return;
	}
	case CPG_DRSPRING: {
		double wrn = A.w - B.w;
		double w_damp = (row.jnt.bias - wrn)*row.jnt.coef;
		row.jnt.bias = wrn + w_damp;
		double j_damp = w_damp*row.jnt.nMass;
		row.jnt.jnAcc += j_damp;
		A.w += j_damp*A.iinv;
		B.w -= j_damp*B.iinv;
		return;
	}
	case CPG_ROTLIMIT: case CPG_RATCHET: {
		if(!row.jnt.bias) return;
		double wr = B.w - A.w;
		double jMax = row.jnt.maxForce*dt;
		double j = -(row.jnt.bias + wr)*row.jnt.nMass;
		double jOld = row.jnt.jnAcc;
		if(row.kind == CPG_RATCHET){
			double ratchet = row.jnt.aux1;
			row.jnt.jnAcc = dclamp((jOld + j)*ratchet, 0.0, jMax*dabs(ratchet))/ratchet;
		} else if(row.jnt.bias < 0.0){
			row.jnt.jnAcc = dclamp(jOld + j, 0.0, jMax);
		} else {
			row.jnt.jnAcc = dclamp(jOld + j, -jMax, 0.0);
		}
		j = row.jnt.jnAcc - jOld;
		A.w -= j*A.iinv;
		B.w += j*B.iinv;
		return;
	}
	case CPG_GEAR: {
		double wr = B.w*row.jnt.aux1 - A.w;
		double jMax = row.jnt.maxForce*dt;
		double j = (row.jnt.bias - wr)*row.jnt.nMass;
		double jOld = row.jnt.jnAcc;
		row.jnt.jnAcc = dclamp(jOld + j, -jMax, jMax);
		j = row.jnt.jnAcc - jOld;
		A.w -= j*A.iinv*row.jnt.aux2;
		B.w += j*B.iinv;
		return;
	}
	default: { /* CPG_MOTOR */
		double wr = B.w - A.w + row.jnt.bias;
		double jMax = row.jnt.maxForce*dt;
		double j = -wr*row.jnt.nMass;
		double jOld = row.jnt.jnAcc;
		row.jnt.jnAcc = dclamp(jOld + j, -jMax, jMax);
		j = row.jnt.jnAcc - jOld;
		A.w -= j*A.iinv;
		B.w += j*B.iinv;
		return;
	}
	}
}

/* Coloured mode, one thread per dynamic body: the warm start (the sweep's
 * first pass) as a gather.  The body takes the cached impulses of its
 * units in colour order, which is the order the coloured sweep applies
 * them to it, with the same operations as row_apply_cached: the result is
 * the sweep's bit for bit, without its twelve or so grid barriers.  The
 * colouring's table gives the unit of each colour on the body. */
__device__ void warm_gather(const cpgSet &s, int w, int x, double &vx, double &vy, double &wv, double minv, double iinv)
{
	const cpgWorld &W = s.world[w];
	double dt_coef = s.params[w].dt_coef;
	unsigned long long m = s.cmask[W.bodyOff + x];
	const int *pos = s.flowPos + 64*(size_t)(W.bodyOff + x);
	const cpgRow *rows = s.rows + W.unitOff;
	BodyRef B;
	B.vx = vx; B.vy = vy; B.w = wv; B.vbx = 0.0; B.vby = 0.0; B.wb = 0.0; B.minv = minv; B.iinv = iinv;
	while(m){
		int c = __ffsll((long long)m) - 1;
		m &= m - 1ull;
		int k = pos[c];
		if(k < 0 || k >= s.tree[w].nunits || k >= W.unitCap) continue;
		const cpgRow &row = rows[k];
		bool isA = (row.a == x), isB = (row.b == x);
		if(row.kind == 0){
			if(row.flags & ROW_FIRST) continue;
			double nx = row.arb.nx, ny = row.arb.ny;
#pragma unroll
			for(int j = 0; j < 2; j++){
				if(j >= row.count) break;
				const cpgRowContact &con = row.arb.c[j];
				double jx = nx*con.jnAcc - ny*con.jtAcc, jy = nx*con.jtAcc + ny*con.jnAcc;
				jx = jx*dt_coef; jy = jy*dt_coef;
				if(isA) apply_impulse(B, -jx, -jy, con.r1x, con.r1y);
				if(isB) apply_impulse(B, jx, jy, con.r2x, con.r2y);
			}
		} else if(row.kind == CPG_DSPRING || row.kind == CPG_DRSPRING){
			continue;
		} else if(row.kind > CPG_SLIDE && row.kind != CPG_GROOVE){
			/* rotary joints: angular impulses only, as row_apply_cached */
			double j = row.jnt.jnAcc*dt_coef;
			if(isA) B.w -= (row.kind == CPG_GEAR) ? j*B.iinv*row.jnt.aux2 : j*B.iinv;
			if(isB) B.w += j*B.iinv;
		} else {
			double jx, jy;
			if(row.kind == CPG_PIVOT || row.kind == CPG_GROOVE){ jx = row.jnt.jx*dt_coef; jy = row.jnt.jy*dt_coef; }
			else { double s_ = row.jnt.jnAcc*dt_coef; jx = row.jnt.nx*s_; jy = row.jnt.ny*s_; }
			if(isA) apply_impulse(B, -jx, -jy, row.jnt.r1x, row.jnt.r1y);
			if(isB) apply_impulse(B, jx, jy, row.jnt.r2x, row.jnt.r2y);
		}
	}
	vx = B.vx; vy = B.vy; wv = B.w;
}

/* one iteration: cpArbiter.c:459-498, cpPivotJoint.c:47-66,
 * cpPinJoint.c:57-75, cpSlideJoint.c:66-89 */
__device__ __forceinline__ void row_apply(cpgRow &row, BodyRef &A, BodyRef &B, double dt)
{
	if(row.kind == 0){
		double nx = row.arb.nx, ny = row.arb.ny;
		double svx = row.arb.svx, svy = row.arb.svy;
		double friction = row.arb.u;
#pragma unroll
		for(int k = 0; k < 2; k++){
			if(k >= row.count) break;
			cpgRowContact &con = row.arb.c[k];
			double nMass = con.nMass;
			double r1x = con.r1x, r1y = con.r1y, r2x = con.r2x, r2y = con.r2y;
			double vb1x = A.vbx + (-r1y)*A.wb, vb1y = A.vby + r1x*A.wb;
			double vb2x = B.vbx + (-r2y)*B.wb, vb2y = B.vby + r2x*B.wb;
			double v1x = A.vx + (-r1y)*A.w, v1y = A.vy + r1x*A.w;
			double v2x = B.vx + (-r2y)*B.w, v2y = B.vy + r2x*B.w;
			double vrx = (v2x - v1x) + svx, vry = (v2y - v1y) + svy;
			double vbn = (vb2x - vb1x)*nx + (vb2y - vb1y)*ny;
			double vrn = vrx*nx + vry*ny;
			double vrt = vrx*(-ny) + vry*nx;
			double jbn = (con.bias - vbn)*nMass;
			double jbnOld = con.jBias;
			con.jBias = dmax0(jbnOld + jbn);
			double jn = -(con.bounce + vrn)*nMass;
			double jnOld = con.jnAcc;
			con.jnAcc = dmax0(jnOld + jn);
			double jtMax = friction*con.jnAcc;
			double jt = -vrt*con.tMass;
			double jtOld = con.jtAcc;
			con.jtAcc = dclamp_sym(jtOld + jt, jtMax);
			double db = con.jBias - jbnOld;
			double bx = nx*db, by = ny*db;
			apply_bias_impulse(A, -bx, -by, r1x, r1y);
			apply_bias_impulse(B, bx, by, r2x, r2y);
			double djn = con.jnAcc - jnOld, djt = con.jtAcc - jtOld;
			double jx = nx*djn - ny*djt, jy = nx*djt + ny*djn;
			apply_impulses(A, B, r1x, r1y, r2x, r2y, jx, jy);
		}
		return;
	}
	if(row.kind > CPG_SLIDE){ row_apply_more(row, A, B, dt); return; }
	if(row.kind == CPG_SLIDE && row.jnt.nx == 0.0 && row.jnt.ny == 0.0) return;
	double v1x = A.vx + (-row.jnt.r1y)*A.w, v1y = A.vy + row.jnt.r1x*A.w;
	double v2x = B.vx + (-row.jnt.r2y)*B.w, v2y = B.vy + row.jnt.r2x*B.w;
	double vrx = v2x - v1x, vry = v2y - v1y;
	if(row.kind == CPG_PIVOT){
		double ex = row.jnt.biasx - vrx, ey = row.jnt.biasy - vry;
		double jx = ex*row.jnt.k11 + ey*row.jnt.k12, jy = ex*row.jnt.k21 + ey*row.jnt.k22;
		double oldx = row.jnt.jx, oldy = row.jnt.jy;
		V2 acc = vclamp(v2(row.jnt.jx + jx, row.jnt.jy + jy), row.jnt.maxForce*dt);
		row.jnt.jx = acc.x; row.jnt.jy = acc.y;
		apply_impulses(A, B, row.jnt.r1x, row.jnt.r1y, row.jnt.r2x, row.jnt.r2y, row.jnt.jx - oldx, row.jnt.jy - oldy);
	} else if(row.kind == CPG_PIN){
		double vrn = vrx*row.jnt.nx + vry*row.jnt.ny;
		double jnMax = row.jnt.maxForce*dt;
		double jn = (row.jnt.bias - vrn)*row.jnt.nMass;
		double jnOld = row.jnt.jnAcc;
		row.jnt.jnAcc = dclamp_sym(jnOld + jn, jnMax);
		jn = row.jnt.jnAcc - jnOld;
		apply_impulses(A, B, row.jnt.r1x, row.jnt.r1y, row.jnt.r2x, row.jnt.r2y, row.jnt.nx*jn, row.jnt.ny*jn);
	} else {
		double vrn = vrx*row.jnt.nx + vry*row.jnt.ny;
		double jn = (row.jnt.bias - vrn)*row.jnt.nMass;
		double jnOld = row.jnt.jnAcc;
		row.jnt.jnAcc = dclamp(jnOld + jn, -row.jnt.maxForce*dt, 0.0);
		jn = row.jnt.jnAcc - jnOld;
		apply_impulses(A, B, row.jnt.r1x, row.jnt.r1y, row.jnt.r2x, row.jnt.r2y, row.jnt.nx*jn, row.jnt.ny*jn);
	}
}

template<bool CG>
__device__ __forceinline__ void solve_row(cpgRow *rows, int k, double *bodies, int pass, double dt_coef, double dt)
{
	cpgRow &row = rows[k];
	BodyRef A = load_pbody<CG>(bodies, row.a);
	BodyRef B = load_pbody<CG>(bodies, row.b);
	if(pass == 0) row_apply_cached(row, A, B, dt_coef);
	else row_apply(row, A, B, dt);
	if(row.flags & ROW_DYN_A) store_pbody(bodies, row.a, A);
	if(row.flags & ROW_DYN_B) store_pbody(bodies, row.b, B);
}

/* ---- four lanes per contact unit ----
 * Within one contact the bias impulse reads and writes only bias
 * velocities (v_bias, w_bias) and the normal and friction impulses only
 * velocities (v, w) (cpArbiter.c:459-498).  A contact unit therefore splits
 * into four independent parts, one per body and kind of velocity, and runs
 * on four lanes: lane q of a quad takes side q & 1 (0: body a, 1: body b)
 * and part q >> 1 (0: velocity, 1: bias velocity).  Each lane performs the
 * reference's operations for its body and part in the reference's order;
 * the two lanes of a part exchange contact-point velocities by shuffle;
 * sign flips are exact (xor of the sign bit) and per-part choices are
 * selects.  Results are bit-identical to one lane per unit.
 *
 * Why: FP64 issue is one warp instruction per 64 cycles per SM
 * sub-partition whatever the number of active lanes, so a sweep level
 * costs its FP64 instruction count per warp: about 37 per contact here
 * against about 90 with one lane per unit.  The clamps of the accumulated
 * impulses are integer compares on the bit patterns (dmax0, dclamp_sym),
 * not FP64 ones.  Joint rows run on lane 0. */
struct QuadRow {
	int body, flags, kind, count;
	double nx, ny, u, svx, svy;
	double rx[2], ry[2], nMass[2], tMass[2], c[2], acc[2], jt[2];
};

__device__ __forceinline__ double dneg_if(double x, bool f)
{
	long long b = __double_as_longlong(x);
	return __longlong_as_double(f ? (b ^ (long long)0x8000000000000000ull) : b);
}

__device__ __forceinline__ void quad_load(QuadRow &q, const cpgRow &row, int lane4)
{
	bool side = (lane4 & 1) != 0, bias = (lane4 & 2) != 0;
	q.kind = row.kind; q.flags = row.flags; q.count = row.count;
	q.body = side ? row.b : row.a;
	if(q.kind != 0) return;
	q.nx = row.arb.nx; q.ny = row.arb.ny; q.u = row.arb.u; q.svx = row.arb.svx; q.svy = row.arb.svy;
#pragma unroll
	for(int k = 0; k < 2; k++){
		if(k >= q.count) break;
		const cpgRowContact &c = row.arb.c[k];
		q.rx[k] = side ? c.r2x : c.r1x; q.ry[k] = side ? c.r2y : c.r1y;
		q.nMass[k] = c.nMass; q.tMass[k] = c.tMass;
		q.c[k] = bias ? c.bias : c.bounce;
		q.acc[k] = bias ? c.jBias : c.jnAcc;
		q.jt[k] = c.jtAcc;
	}
}

/* Warm start (pass 0: cpArbiter.c:441-455) or one iteration of a contact
 * row held in registers; accumulators go back to *row.  FUSED (coloured
 * mode, whose sweep order already differs from the reference's) contracts
 * the multiply-adds of an iteration, the accumulations of the normal and
 * friction impulses included: about 25 FP64 instructions per contact
 * instead of 37.  Without it every operation is the reference's. */
template<bool CG, bool FUSED>
__device__ __forceinline__ void quad_apply(const QuadRow &q, cpgRow *row, double *bodies, int pass, double dt_coef, unsigned qmask, int lane4,
	AdjApp *rec = nullptr)
{
	bool side = (lane4 & 1) != 0, bias = (lane4 & 2) != 0;
	if(pass == 0 && ((q.flags & ROW_FIRST) || bias)) return;
	bool dyn = (q.flags & (side ? ROW_DYN_B : ROW_DYN_A)) != 0;
	double *base = bodies + 8*(size_t)q.body;
	double *bp = base + (bias ? 3 : 0);
	double vx, vy, w, minv, iinv;
	if(CG){ vx = __ldcg(bp); vy = __ldcg(bp + 1); w = __ldcg(bp + 2); minv = __ldcg(base + 6); iinv = __ldcg(base + 7); }
	else { vx = bp[0]; vy = bp[1]; w = bp[2]; minv = base[6]; iinv = base[7]; }
	double nx = q.nx, ny = q.ny;
	if(pass == 0){
#pragma unroll
		for(int k = 0; k < 2; k++){
			if(k >= q.count) break;
			/* j = rotate(n, (jnAcc, jtAcc)) * dt_coef, negated for body a */
			double jx = nx*q.acc[k] - ny*q.jt[k], jy = nx*q.jt[k] + ny*q.acc[k];
			jx = dneg_if(jx*dt_coef, !side); jy = dneg_if(jy*dt_coef, !side);
			vx = vx + jx*minv;
			vy = vy + jy*minv;
			w += iinv*(q.rx[k]*jy - q.ry[k]*jx);
		}
	} else {
#pragma unroll
		for(int k = 0; k < 2; k++){
			if(k >= q.count) break;
			double rx = q.rx[k], ry = q.ry[k];
			double px, py, vn, vt, nxj, nyj;
			double ox, oy, v1x, v1y, v2x, v2y, dx, dy, sx, sy, vrx, vry;
			if(FUSED){ px = __fma_rn(-ry, w, vx); py = __fma_rn(rx, w, vy); }
			else { px = vx + (-ry)*w; py = vy + rx*w; }
			/* contact-point velocity of this lane's body, then of the other */
			ox = __shfl_xor_sync(qmask, px, 1); oy = __shfl_xor_sync(qmask, py, 1);
			v1x = side ? ox : px; v1y = side ? oy : py;
			v2x = side ? px : ox; v2y = side ? py : oy;
			dx = v2x - v1x; dy = v2y - v1y;
			sx = dx + q.svx; sy = dy + q.svy;
			vrx = bias ? dx : sx; vry = bias ? dy : sy;
			if(FUSED){ vn = __fma_rn(vrx, nx, vry*ny); vt = __fma_rn(vry, nx, -(vrx*ny)); }
			else { vn = vrx*nx + vry*ny; vt = vrx*(-ny) + vry*nx; }
			/* velocity: jn = -(bounce + vrn)*nMass; bias: jbn = (bias - vbn)*nMass */
			double y = q.c[k] + dneg_if(vn, bias);
			double old = q.acc[k], jtOld = q.jt[k];
			double acc, jtAcc;
			if(FUSED){
				acc = dmax0(__fma_rn(dneg_if(y, !bias), q.nMass[k], old));
				jtAcc = dclamp_sym(__fma_rn(-vt, q.tMass[k], jtOld), q.u*acc);
			} else {
				double j = dneg_if(y, !bias)*q.nMass[k];
				acc = dmax0(old + j);
				/* friction (used by the velocity lanes only) */
				double jtMax = q.u*acc;
				double jt = -vt*q.tMass[k];
				jtAcc = dclamp_sym(jtOld + jt, jtMax);
			}
			double d = acc - old, djt = jtAcc - jtOld;
			double ax = nx*d, ay = ny*d;
			if(FUSED){ nxj = __fma_rn(-ny, djt, ax); nyj = __fma_rn(nx, djt, ay); }
			else { nxj = ax - ny*djt; nyj = nx*djt + ay; }
			double jx = bias ? ax : nxj, jy = bias ? ay : nyj;
			jx = dneg_if(jx, !side); jy = dneg_if(jy, !side);
			if(rec){
				/* rollout recording: each lane writes its part of the record */
				AdjApp &r = rec[k];
				if(lane4 == 0){ r.jN0 = old; r.jN1 = acc; r.jT0 = jtOld; r.jT1 = jtAcc; r.vrx = vrx; r.vry = vry; r.wA = w; }
				else if(lane4 == 1){ r.wB = w; }
				else if(lane4 == 2){ r.jB0 = old; r.jB1 = acc; r.vbx = vrx; r.vby = vry; r.wbA = w; }
				else { r.wbB = w; }
			}
			if(FUSED){
				vx = __fma_rn(jx, minv, vx);
				vy = __fma_rn(jy, minv, vy);
				w = __fma_rn(iinv, __fma_rn(rx, jy, -(ry*jx)), w);
			} else {
				vx = vx + jx*minv;
				vy = vy + jy*minv;
				w += iinv*(rx*jy - ry*jx);
			}
			if(lane4 == 0){ row->arb.c[k].jnAcc = acc; row->arb.c[k].jtAcc = jtAcc; }
			else if(lane4 == 2){ row->arb.c[k].jBias = acc; }
		}
	}
	if(dyn){ bp[0] = vx; bp[1] = vy; bp[2] = w; }
}

/* ---- two lanes per contact unit ----
 * Lane p of a pair takes part p (0: velocity with the normal and friction
 * impulses, 1: bias velocity with the bias impulse) for both bodies: it
 * computes both contact-point velocities and applies the impulse to both
 * bodies, with the reference's operations in the reference's order, as
 * quad_apply does for one body.  About 50 FP64 instructions per contact
 * lane against 37 on four lanes, but twice the units per warp, so levels
 * of 9 to 16 units (and colours wider than the grid's quads) cost fewer
 * instructions.  Results are bit-identical to the other two layouts. */
struct PairRow {
	int a, b, flags, kind, count;
	double nx, ny, u, svx, svy;
	double r1x[2], r1y[2], r2x[2], r2y[2], nMass[2], tMass[2], c[2], acc[2], jt[2];
};

__device__ __forceinline__ void pair_load(PairRow &q, const cpgRow &row, bool bias)
{
	q.kind = row.kind; q.flags = row.flags; q.count = row.count;
	q.a = row.a; q.b = row.b;
	if(q.kind != 0) return;
	q.nx = row.arb.nx; q.ny = row.arb.ny; q.u = row.arb.u; q.svx = row.arb.svx; q.svy = row.arb.svy;
#pragma unroll
	for(int k = 0; k < 2; k++){
		if(k >= q.count) break;
		const cpgRowContact &c = row.arb.c[k];
		q.r1x[k] = c.r1x; q.r1y[k] = c.r1y; q.r2x[k] = c.r2x; q.r2y[k] = c.r2y;
		q.nMass[k] = c.nMass; q.tMass[k] = c.tMass;
		q.c[k] = bias ? c.bias : c.bounce;
		q.acc[k] = bias ? c.jBias : c.jnAcc;
		q.jt[k] = c.jtAcc;
	}
}

template<bool CG, bool FUSED>
__device__ __forceinline__ void pair_apply(const PairRow &q, cpgRow *row, double *bodies, int pass, double dt_coef, bool bias)
{
	if(pass == 0 && ((q.flags & ROW_FIRST) || bias)) return;
	double *ba = bodies + 8*(size_t)q.a, *bb = bodies + 8*(size_t)q.b;
	double *pa = ba + (bias ? 3 : 0), *pb = bb + (bias ? 3 : 0);
	double avx, avy, aw, am, ai, bvx, bvy, bw, bm, bi;
	if(CG){
		avx = __ldcg(pa); avy = __ldcg(pa + 1); aw = __ldcg(pa + 2); am = __ldcg(ba + 6); ai = __ldcg(ba + 7);
		bvx = __ldcg(pb); bvy = __ldcg(pb + 1); bw = __ldcg(pb + 2); bm = __ldcg(bb + 6); bi = __ldcg(bb + 7);
	} else {
		avx = pa[0]; avy = pa[1]; aw = pa[2]; am = ba[6]; ai = ba[7];
		bvx = pb[0]; bvy = pb[1]; bw = pb[2]; bm = bb[6]; bi = bb[7];
	}
	double nx = q.nx, ny = q.ny;
	if(pass == 0){
#pragma unroll
		for(int k = 0; k < 2; k++){
			if(k >= q.count) break;
			double jx = nx*q.acc[k] - ny*q.jt[k], jy = nx*q.jt[k] + ny*q.acc[k];
			jx = jx*dt_coef; jy = jy*dt_coef;
			avx = avx + (-jx)*am; avy = avy + (-jy)*am;
			aw += ai*(q.r1x[k]*(-jy) - q.r1y[k]*(-jx));
			bvx = bvx + jx*bm; bvy = bvy + jy*bm;
			bw += bi*(q.r2x[k]*jy - q.r2y[k]*jx);
		}
	} else {
#pragma unroll
		for(int k = 0; k < 2; k++){
			if(k >= q.count) break;
			double r1x = q.r1x[k], r1y = q.r1y[k], r2x = q.r2x[k], r2y = q.r2y[k];
			double v1x, v1y, v2x, v2y, vn, vt, nxj, nyj;
			if(FUSED){
				v1x = __fma_rn(-r1y, aw, avx); v1y = __fma_rn(r1x, aw, avy);
				v2x = __fma_rn(-r2y, bw, bvx); v2y = __fma_rn(r2x, bw, bvy);
			} else {
				v1x = avx + (-r1y)*aw; v1y = avy + r1x*aw;
				v2x = bvx + (-r2y)*bw; v2y = bvy + r2x*bw;
			}
			double dx = v2x - v1x, dy = v2y - v1y;
			double sx = dx + q.svx, sy = dy + q.svy;
			double vrx = bias ? dx : sx, vry = bias ? dy : sy;
			if(FUSED){ vn = __fma_rn(vrx, nx, vry*ny); vt = __fma_rn(vry, nx, -(vrx*ny)); }
			else { vn = vrx*nx + vry*ny; vt = vrx*(-ny) + vry*nx; }
			double y = q.c[k] + dneg_if(vn, bias);
			double old = q.acc[k], jtOld = q.jt[k];
			double acc, jtAcc;
			if(FUSED){
				acc = dmax0(__fma_rn(dneg_if(y, !bias), q.nMass[k], old));
				jtAcc = dclamp_sym(__fma_rn(-vt, q.tMass[k], jtOld), q.u*acc);
			} else {
				double j = dneg_if(y, !bias)*q.nMass[k];
				acc = dmax0(old + j);
				double jtMax = q.u*acc;
				double jt = -vt*q.tMass[k];
				jtAcc = dclamp_sym(jtOld + jt, jtMax);
			}
			double d = acc - old, djt = jtAcc - jtOld;
			double ax = nx*d, ay = ny*d;
			if(FUSED){ nxj = __fma_rn(-ny, djt, ax); nyj = __fma_rn(nx, djt, ay); }
			else { nxj = ax - ny*djt; nyj = nx*djt + ay; }
			double jx = bias ? ax : nxj, jy = bias ? ay : nyj;
			if(FUSED){
				avx = __fma_rn(-jx, am, avx); avy = __fma_rn(-jy, am, avy);
				aw = __fma_rn(ai, __fma_rn(r1x, -jy, -(r1y*(-jx))), aw);
				bvx = __fma_rn(jx, bm, bvx); bvy = __fma_rn(jy, bm, bvy);
				bw = __fma_rn(bi, __fma_rn(r2x, jy, -(r2y*jx)), bw);
			} else {
				avx = avx + (-jx)*am; avy = avy + (-jy)*am;
				aw += ai*(r1x*(-jy) - r1y*(-jx));
				bvx = bvx + jx*bm; bvy = bvy + jy*bm;
				bw += bi*(r2x*jy - r2y*jx);
			}
			if(!bias){ row->arb.c[k].jnAcc = acc; row->arb.c[k].jtAcc = jtAcc; }
			else row->arb.c[k].jBias = acc;
		}
	}
	if(q.flags & ROW_DYN_A){ pa[0] = avx; pa[1] = avy; pa[2] = aw; }
	if(q.flags & ROW_DYN_B){ pb[0] = bvx; pb[1] = bvy; pb[2] = bw; }
}

/* Layout of a level of U units for a block of `nt` threads: the cheapest
 * in FP64 warp instructions per contact of four lanes (37 per round of
 * nt/4 units), two lanes (50 per round of nt/2) and one lane (90 per
 * round of nt).  0: four, 1: two, 2: one. */
__device__ __forceinline__ int level_layout(int U, int nt, bool many)
{
	int w4 = (4*U + 31) >> 5, w2 = (2*U + 31) >> 5, w1 = (U + 31) >> 5;
	int r4 = (4*U + nt - 1)/nt, r2 = (2*U + nt - 1)/nt, r1 = (U + nt - 1)/nt;
	long c4, c2, c1;
	if(many){
		/* many worlds share each sub-partition's FP64 pipe: fewest warp
		 * instructions (ties: fewest rounds) */
		c4 = (long)w4*37*1024 + r4; c2 = (long)w2*50*1024 + r2; c1 = (long)w1*90*1024 + r1;
	} else {
		/* few worlds: the level's dependent chain, rounds x per-lane count */
		c4 = (long)r4*37*1024 + w4; c2 = (long)r2*50*1024 + w2; c1 = (long)r1*90*1024 + w1;
	}
	return (c4 <= c2 && c4 <= c1) ? 0 : (c2 <= c1 ? 1 : 2);
}

extern __shared__ double sbody[];

/* Warm start (pass 0) and `iterations` sweeps, level by level; one block
 * per world.  Worlds of at most `stagedMax` bodies keep their packed body
 * state in shared memory for the whole solve. */
__global__ void __launch_bounds__(256, 2) k_solve(cpgSet s, int stagedMax)
{
	/* largest worlds first: their long level chains start at once */
	int w = s.worldOrder[blockIdx.x];
	const cpgParams &P = s.params[w];
	if(!P.active) return;
	const cpgWorld &W = s.world[w];
	const cpgTree &T = s.tree[w];
	int nunits = T.nunits, nlev = T.nlevels;
	if(nunits > W.unitCap) return;
	bool staged = W.nbodies <= stagedMax;
	double *gb = s.pbody + 8*(size_t)W.bodyOff;
	if(staged){
		for(int i = threadIdx.x; i < 8*W.nbodies; i += blockDim.x) sbody[i] = gb[i];
		__syncthreads();
	}
	double *bodies = staged ? sbody : gb;
	const int *start = s.levelStart + W.unitOff + w;
	cpgRow *rows = s.rows + W.unitOff;
	int lane4 = threadIdx.x & 3, nq = blockDim.x >> 2;
	unsigned qmask = 0xFu << (threadIdx.x & 28);
	/* rollout recording: the rows of this world in the tape */
	AdjApp *tapeApp = nullptr;
	if(s.tape.on && s.tape.app){
		const int *off = s.tape.rowOff + (size_t)s.tape.step*(s.nworlds + 1);
		/* past the tape's capacity nothing is recorded: the host grows the
		 * tape and replays the segment */
		if(off[w + 1] <= s.tape.rowCap) tapeApp = (AdjApp *)s.tape.app + (size_t)off[w]*P.iterations*2;
	}
	int nt = blockDim.x;
	bool many = s.solveLayout == 1 || (s.solveLayout == 0 && s.nworlds >= 152);
	bool recording = (s.tape.on && s.tape.app) || s.solveLayout == 3;
	for(int pass = 0; pass <= P.iterations; pass++){
		for(int l = 0; l < nlev; l++){
			int b0 = start[l], e = start[l + 1];
			/* the recording pass writes its records from four lanes */
			int lay = recording ? 0 : level_layout(e - b0, nt, many);
			if(lay == 0){
				for(int k = b0 + (threadIdx.x >> 2); k < e; k += nq){
					QuadRow q;
					quad_load(q, rows[k], lane4);
					AdjApp *rec = (tapeApp && pass > 0) ? tapeApp + ((size_t)k*P.iterations + (pass - 1))*2 : nullptr;
					if(q.kind == 0) quad_apply<false, false>(q, rows + k, bodies, pass, P.dt_coef, qmask, lane4, rec);
					else if(lane4 == 0){
						if(tapeApp) atomicOr(&s.tape.cursor[3], 1);   /* joints are not differentiated */
						solve_row<false>(rows, k, bodies, pass, P.dt_coef, P.dt);
					}
				}
			} else if(lay == 1){
				bool bias = (threadIdx.x & 1) != 0;
				for(int k = b0 + (threadIdx.x >> 1); k < e; k += nt >> 1){
					PairRow q;
					pair_load(q, rows[k], bias);
					if(q.kind == 0) pair_apply<false, false>(q, rows + k, bodies, pass, P.dt_coef, bias);
					else if(!bias) solve_row<false>(rows, k, bodies, pass, P.dt_coef, P.dt);
				}
			} else {
				for(int k = b0 + threadIdx.x; k < e; k += nt) solve_row<false>(rows, k, bodies, pass, P.dt_coef, P.dt);
			}
			__syncthreads();
		}
	}
	if(staged){
		for(int i = threadIdx.x; i < 8*W.nbodies; i += blockDim.x) gb[i] = sbody[i];
	}
}

/* The solver iterations of recorded steps, recomputed for the rollout's
 * reverse pass (one block per world and step of a segment: the steps are
 * independent given what the forward recorded).  Each block starts from
 * the step's recorded solver input, the velocities after integration and
 * the pre-step rows, runs the same four-lane sweep as k_solve (bit for bit
 * the forward's solve) and writes the per-iteration application records.
 * The rows it updates are a copy; bodies are staged like k_solve's. */
__global__ void __launch_bounds__(256, 2) k_replay_solve(cpgSet s, cpgAdj a, int stagedMax)
{
	int w = s.worldOrder[blockIdx.x], t = blockIdx.y;
	const cpgTape &tp = s.tape;
	int nw = s.nworlds;
	const cpgParams P = tp.params[(size_t)t*nw + w];
	if(!P.active) return;
	const cpgWorld &W = s.world[w];
	int ro = tp.rowOff[(size_t)t*(nw + 1) + w];
	int n = tp.rowOff[(size_t)t*(nw + 1) + w + 1] - ro;
	int lo = tp.levOff[(size_t)t*(nw + 1) + w];
	int nlev = tp.levOff[(size_t)t*(nw + 1) + w + 1] - lo - 1;
	if(ro + n > tp.rowCap || nlev < 0) return;
	const int *start = tp.levels + lo;
	cpgRow *rows = a.srows + ro;
	int nbw = W.nbodies, bo = W.bodyOff, nb = s.totalBodies;
	bool staged = nbw <= stagedMax;
	double *bodies = staged ? sbody : a.sbodies + 8*((size_t)t*nb + bo);
	const double *vel = tp.vel + (size_t)t*3*nb;
	for(int k = threadIdx.x; k < n; k += blockDim.x) rows[k] = tp.rows[ro + k];
	for(int i = threadIdx.x; i < nbw; i += blockDim.x){
		int g = bo + i;
		double *b = bodies + 8*(size_t)i;
		b[0] = vel[g]; b[1] = vel[nb + g]; b[2] = vel[2*(size_t)nb + g];
		b[3] = 0.0; b[4] = 0.0; b[5] = 0.0;
		b[6] = s.minv[g]; b[7] = s.iinv[g];
	}
	__syncthreads();
	AdjApp *tapeApp = (AdjApp *)tp.app + (size_t)ro*P.iterations*2;
	int lane4 = threadIdx.x & 3, nq = blockDim.x >> 2;
	unsigned qmask = 0xFu << (threadIdx.x & 28);
	for(int pass = 0; pass <= P.iterations; pass++){
		for(int l = 0; l < nlev; l++){
			int e = start[l + 1];
			for(int k = start[l] + (threadIdx.x >> 2); k < e; k += nq){
				QuadRow q;
				quad_load(q, rows[k], lane4);
				AdjApp *rec = pass > 0 ? tapeApp + ((size_t)k*P.iterations + (pass - 1))*2 : nullptr;
				if(q.kind == 0) quad_apply<false, false>(q, rows + k, bodies, pass, P.dt_coef, qmask, lane4, rec);
				else if(lane4 == 0) solve_row<false>(rows, k, bodies, pass, P.dt_coef, P.dt);
			}
			__syncthreads();
		}
	}
}

/* Rows back to the arbiter table and the joint records (the warm-start
 * state of the next step), packed bodies back to the body arrays. */
__global__ void k_writeback(cpgSet s)
{
	int w = blockIdx.y;
	if(!s.params[w].active) return;
	const cpgWorld &W = s.world[w];
	const cpgTree &T = s.tree[w];
	int nunits = T.nunits;
	if(nunits > W.unitCap) return;
	for(int k = blockIdx.x*blockDim.x + threadIdx.x; k < nunits; k += gridDim.x*blockDim.x){
		const cpgRow &row = s.rows[W.unitOff + k];
		if(row.kind == 0){
			cpgArb &arb = s.arbs[row.src];
			for(int c = 0; c < row.count; c++){
				const cpgRowContact &rc = row.arb.c[c];
				cpgContact &con = arb.c[c];
				con.nMass = rc.nMass; con.tMass = rc.tMass; con.bounce = rc.bounce; con.bias = rc.bias;
				con.jnAcc = rc.jnAcc; con.jtAcc = rc.jtAcc; con.jBias = rc.jBias;
			}
		} else {
			cpgJoint &j = s.joints[W.consOff + row.src];
			j.r1x = row.jnt.r1x; j.r1y = row.jnt.r1y; j.r2x = row.jnt.r2x; j.r2y = row.jnt.r2y;
			if(row.kind == CPG_PIVOT || row.kind == CPG_GROOVE){
				j.k11 = row.jnt.k11; j.k12 = row.jnt.k12; j.k21 = row.jnt.k21; j.k22 = row.jnt.k22;
				j.jx = row.jnt.jx; j.jy = row.jnt.jy; j.biasx = row.jnt.biasx; j.biasy = row.jnt.biasy;
				j.nx = row.jnt.nx; j.ny = row.jnt.ny; j.clamp = row.jnt.clamp;
			} else {
				j.nx = row.jnt.nx; j.ny = row.jnt.ny; j.nMass = row.jnt.nMass; j.jnAcc = row.jnt.jnAcc; j.bias = row.jnt.bias;
				j.coef = row.jnt.coef;
			}
		}
	}
}

__global__ void k_unpack_bodies(cpgSet s)
{
	int g = blockIdx.x*blockDim.x + threadIdx.x;
	if(g >= s.totalBodies) return;
	int w = s.bworld[g];
	if(!s.params[w].active || s.btype[g] != CPG_DYNAMIC) return;
	const double2 *pb = (const double2 *)(s.pbody + 8*(size_t)g);
	double2 x0 = pb[0], x1 = pb[1], x2 = pb[2];
	s.vx[g] = x0.x; s.vy[g] = x0.y; s.w[g] = x1.x;
	s.vbx[g] = x1.y; s.vby[g] = x2.x; s.wb[g] = x2.y;
}

/* Aggregate per-world bookkeeping for the host (one block). */
__global__ void k_stats(cpgSet s)
{
	__shared__ int err, pairMax, nodeMax, candMax, levMax, ncand, narb, moved;
	if(threadIdx.x == 0){ err = 0; pairMax = 0; nodeMax = 0; candMax = 0; levMax = 0; ncand = 0; narb = 0; moved = 0; }
	__syncthreads();
	for(int w = threadIdx.x; w < s.nworlds; w += blockDim.x){
		const cpgTree &T = s.tree[w];
		const cpgWorld &W = s.world[w];
		atomicOr(&err, T.error);
		atomicMax(&pairMax, (int)((long long)T.pairTop*1000/(W.pairCap > 0 ? W.pairCap : 1)));
		atomicMax(&nodeMax, (int)((long long)T.nodeTop*1000/(W.nodeCap > 0 ? W.nodeCap : 1)));
		atomicMax(&candMax, (int)((long long)T.ncand*1000/(W.candCap > 0 ? W.candCap : 1)));
		atomicMax(&levMax, T.nlevels);
		atomicAdd(&ncand, T.ncand);
		atomicAdd(&narb, T.narb);
		atomicAdd(&moved, T.moved);
	}
	__syncthreads();
	if(threadIdx.x == 0){
		s.stats[0] = err; s.stats[1] = pairMax; s.stats[2] = nodeMax; s.stats[4] = ncand;
		s.stats[5] = narb; s.stats[6] = levMax; s.stats[7] = candMax; s.stats[8] = moved;
	}
}

/* Overwrite the accumulated impulses of one world's last solve list with
 * records in its order (4 doubles each: jnAcc, jtAcc of contacts 0, 1;
 * 2 ints each: the shapes the record belongs to).  A record whose shapes
 * differ from the listed arbiter's is skipped and counted in *mismatch. */
__global__ void k_set_arb_impulses(cpgSet s, int w, const double *imp, const int *pairs, int n, int *mismatch)
{
	int i = blockIdx.x*blockDim.x + threadIdx.x;
	const cpgTree &T = s.tree[w];
	if(i >= n || i >= T.narb) return;
	cpgArb &arb = s.arbs[s.arbList[s.world[w].candOff + i]];
	if(arb.a != pairs[2*i] || arb.b != pairs[2*i + 1]){ atomicAdd(mismatch, 1); return; }
	for(int k = 0; k < arb.count && k < 2; k++){
		arb.c[k].jnAcc = imp[4*i + 2*k];
		arb.c[k].jtAcc = imp[4*i + 2*k + 1];
	}
}

extern "C" int cpg_launch_set_arb_impulses(const cpgSet *s, int w, const double *imp, const int *pairs, int n, int *mismatch, void *stream)
{
	if(n <= 0) return 0;
	LAUNCH(k_set_arb_impulses<<<(n + 127)/128, 128, 0, (cudaStream_t)stream>>>(*s, w, imp, pairs, n, mismatch));
	return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

/* Contact quality of one world after a step, from its solver rows and
 * final velocities (all contacts of all arbiter rows):
 *   normal residual: |vn + bounce| where the accumulated normal impulse is
 *     positive, else the approach speed max(0, -(vn + bounce)) -- the
 *     complementarity the sequential impulses converge to
 *     (cpArbiter.c:459-498);
 *   friction residual: |vt| for a contact inside the friction cone
 *     (|jt| < u jn), else the slip along the friction impulse
 *     max(0, vt sign(jt)) (friction must oppose sliding);
 *   penetration: max(0, -d'), d' the contact's separation along n after
 *     the next position update, d + dt (vn + vbn): d at the step's
 *     positions (cpArbiterGetDepth, cpArbiter.c:90-98), vn and vbn the
 *     relative normal velocity and bias velocity the solve left.
 * acc: [0] sum of squared normal residuals, [1] of friction residuals,
 * [2] contacts, [3] largest penetration (as the bits of a non-negative
 * double, so that integer max orders them). */
__global__ void k_contact_quality(cpgSet s, int w, double dt, double *acc)
{
	const cpgWorld &W = s.world[w];
	const cpgTree &T = s.tree[w];
	int nunits = T.nunits;
	if(nunits > W.unitCap) return;
	double sn = 0.0, stt = 0.0, cnt = 0.0, pen = 0.0;
	for(int k = blockIdx.x*blockDim.x + threadIdx.x; k < nunits; k += gridDim.x*blockDim.x){
		const cpgRow &row = s.rows[W.unitOff + k];
		if(row.kind != 0) continue;
		int ga = W.bodyOff + row.a, gb = W.bodyOff + row.b;
		double nx = row.arb.nx, ny = row.arb.ny, u = row.arb.u;
		for(int c = 0; c < row.count && c < 2; c++){
			const cpgRowContact &rc = row.arb.c[c];
			double v1x = s.vx[ga] + (-rc.r1y)*s.w[ga], v1y = s.vy[ga] + rc.r1x*s.w[ga];
			double v2x = s.vx[gb] + (-rc.r2y)*s.w[gb], v2y = s.vy[gb] + rc.r2x*s.w[gb];
			double vrx = (v2x - v1x) + row.arb.svx, vry = (v2y - v1y) + row.arb.svy;
			double vn = vrx*nx + vry*ny, vt = vrx*(-ny) + vry*nx;
			double rn = vn + rc.bounce;
			double resn = rc.jnAcc > 0.0 ? fabs(rn) : fmax(0.0, -rn);
			double rest = fabs(rc.jtAcc) < u*rc.jnAcc ? fabs(vt) : fmax(0.0, rc.jtAcc > 0.0 ? vt : (rc.jtAcc < 0.0 ? -vt : 0.0));
			double dx = (rc.r2x - rc.r1x) + (s.px[gb] - s.px[ga]), dy = (rc.r2y - rc.r1y) + (s.py[gb] - s.py[ga]);
			double b1x = s.vbx[ga] + (-rc.r1y)*s.wb[ga], b1y = s.vby[ga] + rc.r1x*s.wb[ga];
			double b2x = s.vbx[gb] + (-rc.r2y)*s.wb[gb], b2y = s.vby[gb] + rc.r2x*s.wb[gb];
			double vbn = (b2x - b1x)*nx + (b2y - b1y)*ny;
			double d = (dx*nx + dy*ny) + dt*(((v2x - v1x)*nx + (v2y - v1y)*ny) + vbn);
			sn += resn*resn; stt += rest*rest; cnt += 1.0;
			pen = fmax(pen, -d);
		}
	}
	for(int o = 16; o > 0; o >>= 1){
		sn += __shfl_down_sync(0xffffffffu, sn, o);
		stt += __shfl_down_sync(0xffffffffu, stt, o);
		cnt += __shfl_down_sync(0xffffffffu, cnt, o);
		pen = fmax(pen, __shfl_down_sync(0xffffffffu, pen, o));
	}
	if((threadIdx.x & 31) == 0 && cnt > 0.0){
		atomicAdd(&acc[0], sn); atomicAdd(&acc[1], stt); atomicAdd(&acc[2], cnt);
		atomicMax((unsigned long long *)&acc[3], (unsigned long long)__double_as_longlong(fmax(pen, 0.0)));
	}
}

/* The public view of world w's first n bodies, 8 doubles each, as the
 * getters compute it (cpBody.c): position cpTransformPoint(transform,
 * cpvzero), velocity, angle, angular velocity, rotation (transform.a,
 * transform.b). */
__global__ void k_body_states(cpgSet s, int w, double *out, int n)
{
	int i = blockIdx.x*blockDim.x + threadIdx.x;
	if(i >= n) return;
	int g = s.world[w].bodyOff + i;
	double ta = s.ta[g], tb = s.tb[g], tc = s.tc[g], td = s.td[g];
	double *o = out + 8*(size_t)i;
	o[0] = ta*0.0 + tc*0.0 + s.ttx[g];
	o[1] = tb*0.0 + td*0.0 + s.tty[g];
	o[2] = s.vx[g]; o[3] = s.vy[g];
	o[4] = s.ang[g]; o[5] = s.w[g];
	o[6] = ta; o[7] = tb;
}

extern "C" int cpg_launch_contact_quality(const cpgSet *s, int w, double dt, double *acc, void *stream)
{
	cudaStream_t st = (cudaStream_t)stream;
	cudaMemsetAsync(acc, 0, 4*sizeof(double), st);
	LAUNCH(k_contact_quality<<<152*2, 256, 0, st>>>(*s, w, dt, acc));
	return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

/* Copy one world's solve list of arbiters into a contiguous buffer. */
/* Arbiter records by table slot (host callbacks of collision handlers). */
__global__ void k_gather_slots(cpgSet s, const int *slots, cpgArb *out, int n)
{
	for(int i = blockIdx.x*blockDim.x + threadIdx.x; i < n; i += gridDim.x*blockDim.x) out[i] = s.arbs[slots[i]];
}

/* Records changed by the host's callbacks back into their slots. */
__global__ void k_put_arbs(cpgSet s, const int *slots, const cpgArb *recs, int n)
{
	for(int i = blockIdx.x*blockDim.x + threadIdx.x; i < n; i += gridDim.x*blockDim.x) s.arbs[slots[i]] = recs[i];
}

/* Slots of the cached arbiters of one shape of world 0 (cpSpaceFilterArbiters
 * on removal, cpSpace.c:481-521); the count may pass cap. */
__global__ void k_shape_arbs(cpgSet s, int shape, int *slots, int *count, int cap)
{
	for(int i = blockIdx.x*blockDim.x + threadIdx.x; i < s.arbCap; i += gridDim.x*blockDim.x){
		if(s.keys[i] <= CPG_KEY_TOMB) continue;
		const cpgArb &a = s.arbs[i];
		if(a.world != 0 || (a.a != shape && a.b != shape) || (a.pad & CPG_ARB_ASLEEP)) continue;
		int k = atomicAdd(count, 1);
		if(k < cap) slots[k] = i;
	}
}

__global__ void k_gather_arbs(cpgSet s, int w, cpgArb *out, int n)
{
	int i = blockIdx.x*blockDim.x + threadIdx.x;
	if(i >= n) return;
	out[i] = s.arbs[s.arbList[s.world[w].candOff + i]];
}

/* The shape pairs of a world's arbiter list, in info order (the contact
 * graph's needs: 8 bytes per arbiter instead of the whole record). */
__global__ void k_gather_pairs(cpgSet s, int w, int2 *out, int n)
{
	int i = blockIdx.x*blockDim.x + threadIdx.x;
	if(i >= n) return;
	const cpgArb &a = s.arbs[s.arbList[s.world[w].candOff + i]];
	out[i] = make_int2(a.a, a.b);
}

/* Whole records by table key (arbiters out of the list: those held by
 * sleeping bodies); a missing key gives a record with shape -1. */
__global__ void k_gather_keys(cpgSet s, const unsigned long long *keys, cpgArb *out, int n)
{
	int i = blockIdx.x*blockDim.x + threadIdx.x;
	if(i >= n) return;
	int slot = arb_find(s, keys[i]);
	if(slot >= 0) out[i] = s.arbs[slot];
	else { out[i].a = -1; out[i].b = -1; }
}

/* ------------------------------------------------------------------ */
/* Coloured mode (single-world sets): sweep-and-prune, colouring, solve */

/* Sweep axis: the one along which the shape centres spread more (their
 * variance), so that a sweep visits fewer boxes.  One block. */
/* ---- sweep order: one cooperative launch per step ----
 *
 * The sweep order is the dynamic shapes sorted by (left-edge key, shape
 * index), a unique order.  Between steps it barely changes, so the keys
 * are first recomputed in the previous order as 64-bit (key << 32 | shape)
 * values and repaired by odd-even transposition rounds (compare-exchange
 * of (2i, 2i+1), then of (2i+1, 2i+2)); a round with no exchange leaves the
 * keys sorted.  When SAP_REPAIR_ROUNDS rounds do not finish (first step,
 * axis change, fast motion), a stable LSD radix sort by the 32-bit key from
 * shape-index order gives the same order.  Then the boxes are gathered in
 * sweep order, and the sweep axis for the next step is chosen: the axis
 * along which box centres have the larger variance (FP32 sums per block
 * in a fixed order, then over blocks in block order, so the choice is
 * deterministic).  Any axis gives the same pair set. */
#define SAP_THREADS 256
#define SAP_REPAIR_ROUNDS 8

__device__ __forceinline__ unsigned sap_lo_key(const cpgSet &s, int g, int axis)
{
	return float_order_key(__double2float_rd(axis ? s.bbb[g] : s.bbl[g]));
}

__device__ __forceinline__ unsigned sap_hi_key(const cpgSet &s, int g, int axis)
{
	return float_order_key(__double2float_ru(axis ? s.bbt[g] : s.bbr[g]));
}

/* One stable LSD pass over 8 bits with the whole grid: block histograms,
 * per-digit prefixes over blocks (one warp per digit), digit bases, then a
 * stable scatter of each block's contiguous range in sub-tiles.  Data other
 * blocks wrote in this launch is read with __ldcg. */
__device__ void sap_radix_pass(cg::grid_group &grid, const unsigned *kin, const int *vin, unsigned *kout, int *vout,
	int n, int shift, unsigned *hist, unsigned *rowTot)
{
	__shared__ unsigned shHist[256], shBase[256], shTot[256];
	__shared__ unsigned shWarp[SAP_THREADS/32][256];
	int nblk = gridDim.x, b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	int per = (n + nblk - 1)/nblk;
	int lo = b*per, hi = min(n, lo + per);
	shHist[tid] = 0u;
	for(int w2 = 0; w2 < SAP_THREADS/32; w2++) shWarp[w2][tid] = 0u;
	__syncthreads();
	for(int i = lo + tid; i < hi; i += SAP_THREADS) atomicAdd(&shHist[(__ldcg(&kin[i]) >> shift) & 0xFFu], 1u);
	__syncthreads();
	hist[tid*nblk + b] = shHist[tid];
	grid.sync();
	int gw = (b*SAP_THREADS + tid) >> 5, nw = (nblk*SAP_THREADS) >> 5;
	for(int d = gw; d < 256; d += nw){
		unsigned carry = 0u;
		for(int c0 = 0; c0 < nblk; c0 += 32){
			int j = c0 + lane;
			unsigned v = (j < nblk) ? __ldcg(&hist[d*nblk + j]) : 0u;
			unsigned x = v;
			for(int o = 1; o < 32; o <<= 1){
				unsigned y = __shfl_up_sync(0xffffffffu, x, o);
				if(lane >= o) x += y;
			}
			if(j < nblk) hist[d*nblk + j] = carry + x - v;
			carry += __shfl_sync(0xffffffffu, x, 31);
		}
		if(lane == 0) rowTot[d] = carry;
	}
	grid.sync();
	/* digit bases: exclusive scan of the 256 totals (every block) */
	{
		unsigned v = __ldcg(&rowTot[tid]);
		unsigned x = v;
		for(int o = 1; o < 32; o <<= 1){
			unsigned y = __shfl_up_sync(0xffffffffu, x, o);
			if(lane >= o) x += y;
		}
		if(lane == 31) shTot[warp] = x;
		__syncthreads();
		unsigned wp = 0u;
		for(int w2 = 0; w2 < warp; w2++) wp += shTot[w2];
		shBase[tid] = wp + x - v + __ldcg(&hist[tid*nblk + b]);
		__syncthreads();
	}
	for(int t0 = lo; t0 < hi; t0 += SAP_THREADS){
		int i = t0 + tid;
		bool valid = i < hi;
		unsigned key = valid ? __ldcg(&kin[i]) : 0u;
		unsigned d = valid ? ((key >> shift) & 0xFFu) : 256u;
		unsigned peers = __match_any_sync(0xffffffffu, d);
		unsigned rank = __popc(peers & ((1u << lane) - 1u));
		if(valid && rank == 0) shWarp[warp][d] = __popc(peers);
		__syncthreads();
		{
			unsigned acc = 0u;
			for(int w2 = 0; w2 < SAP_THREADS/32; w2++){ unsigned t = shWarp[w2][tid]; shWarp[w2][tid] = acc; acc += t; }
			shTot[tid] = acc;
		}
		__syncthreads();
		if(valid){
			unsigned pos = shBase[d] + shWarp[warp][d] + rank;
			kout[pos] = key;
			vout[pos] = __ldcg(&vin[i]);
		}
		__syncthreads();
		shBase[tid] += shTot[tid];
		for(int w2 = 0; w2 < SAP_THREADS/32; w2++) shWarp[w2][tid] = 0u;
		__syncthreads();
	}
	grid.sync();
}

__global__ void __launch_bounds__(SAP_THREADS, 1) k_sap_sort(cpgSet s, int w)
{
	cg::grid_group grid = cg::this_grid();
	__shared__ float red[4][SAP_THREADS/32];
	const cpgWorld &W = s.world[w];
	int n = W.ndynShapes;
	int gtid = blockIdx.x*SAP_THREADS + threadIdx.x, gsz = gridDim.x*SAP_THREADS;
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	int *cc = s.colorCursor;
	int axis = cc[8];
	bool have = (cc[10] == n + 1) && (cc[11] == axis);
	unsigned long long *K = s.sortK64;
	unsigned *KA = s.sortKA;
	int *VA = s.sortVA;
	if(gtid < 2*SAP_REPAIR_ROUNDS) cc[16 + gtid] = 0;
	grid.sync();
	bool sorted = false;
	if(have){
		for(int i = gtid; i < n; i += gsz){
			int sh = VA[i];
			int g = W.shapeOff + sh;
			K[i] = ((unsigned long long)sap_lo_key(s, g, axis) << 32) | (unsigned)sh;
			s.rkeys[sh] = sap_hi_key(s, g, axis);
		}
		grid.sync();
		for(int round = 0; round < SAP_REPAIR_ROUNDS && !sorted; round++){
			for(int phase = 0; phase < 2; phase++){
				int swaps = 0;
				for(int j = gtid; 2*j + phase + 1 < n; j += gsz){
					int a = 2*j + phase;
					unsigned long long ka = __ldcg(&K[a]), kb = __ldcg(&K[a + 1]);
					if(ka > kb){ K[a] = kb; K[a + 1] = ka; swaps++; }
				}
				swaps = __reduce_add_sync(0xffffffffu, swaps);
				if(lane == 0 && swaps) atomicAdd(&cc[16 + 2*round + phase], swaps);
				grid.sync();
			}
			sorted = (__ldcg(&cc[16 + 2*round]) == 0) && (__ldcg(&cc[16 + 2*round + 1]) == 0);
		}
		if(sorted){
			for(int i = gtid; i < n; i += gsz){
				unsigned long long k = __ldcg(&K[i]);
				KA[i] = (unsigned)(k >> 32);
				VA[i] = (int)(unsigned)(k & 0xFFFFFFFFull);
			}
		}
	}
	if(!sorted){
		for(int k = gtid; k < n; k += gsz){
			int sh = s.dynShapes[W.dynShapeOff + k];
			int g = W.shapeOff + sh;
			KA[k] = sap_lo_key(s, g, axis);
			VA[k] = sh;
			s.rkeys[sh] = sap_hi_key(s, g, axis);
		}
		grid.sync();
		unsigned *hist = s.rsHist, *rowTot = s.rsHist + 256*CPG_SORT_MAX_BLOCKS;
		sap_radix_pass(grid, s.sortKA, s.sortVA, s.sortKB, s.sortVB, n, 0, hist, rowTot);
		sap_radix_pass(grid, s.sortKB, s.sortVB, s.sortKA, s.sortVA, n, 8, hist, rowTot);
		sap_radix_pass(grid, s.sortKA, s.sortVA, s.sortKB, s.sortVB, n, 16, hist, rowTot);
		sap_radix_pass(grid, s.sortKB, s.sortVB, s.sortKA, s.sortVA, n, 24, hist, rowTot);
	} else {
		grid.sync();
	}
	/* boxes in sweep order, and the centre sums for the next axis */
	float sx = 0.0f, sxx = 0.0f, sy = 0.0f, syy = 0.0f;
	for(int k = gtid; k < n; k += gsz){
		int g = W.shapeOff + __ldcg(&VA[k]);
		double l = s.bbl[g], b = s.bbb[g], r = s.bbr[g], t = s.bbt[g];
		longlong4_32a kb4;
		kb4.x = okey(l); kb4.y = okey(b); kb4.z = okey(r); kb4.w = okey(t);
		((longlong4_32a *)s.sapBB)[k] = kb4;
		float cx = 0.5f*((float)l + (float)r), cy = 0.5f*((float)b + (float)t);
		sx += cx; sxx += cx*cx; sy += cy; syy += cy*cy;
	}
	for(int o = 16; o > 0; o >>= 1){
		sx += __shfl_down_sync(0xffffffffu, sx, o); sxx += __shfl_down_sync(0xffffffffu, sxx, o);
		sy += __shfl_down_sync(0xffffffffu, sy, o); syy += __shfl_down_sync(0xffffffffu, syy, o);
	}
	if(lane == 0){ red[0][warp] = sx; red[1][warp] = sxx; red[2][warp] = sy; red[3][warp] = syy; }
	__syncthreads();
	if(threadIdx.x == 0){
		float a = 0.0f, bb = 0.0f, c = 0.0f, d = 0.0f;
		for(int i = 0; i < SAP_THREADS/32; i++){ a += red[0][i]; bb += red[1][i]; c += red[2][i]; d += red[3][i]; }
		float *part = s.sapPart + 4*blockIdx.x;
		part[0] = a; part[1] = bb; part[2] = c; part[3] = d;
	}
	grid.sync();
	if(gtid == 0){
		float a = 0.0f, bb = 0.0f, c = 0.0f, d = 0.0f;
		for(int i = 0; i < (int)gridDim.x; i++){
			const float *part = s.sapPart + 4*i;
			a += __ldcg(part); bb += __ldcg(part + 1); c += __ldcg(part + 2); d += __ldcg(part + 3);
		}
		float nn = n > 0 ? (float)n : 1.0f;
		float vx = bb/nn - (a/nn)*(a/nn), vy = d/nn - (c/nn)*(c/nn);
		cc[8] = (vy > vx) ? 1 : 0;
		cc[10] = n + 1;
		cc[11] = axis;
	}
}

/* One warp per sorted shape: lane 0 queries the static tree, all lanes
 * sweep.  Count pass, then (after the scan) the emit pass writes the pairs
 * at deterministic positions: static hits first, then sweep hits in box
 * order. */
__global__ void k_sap_count(cpgSet s, int w)
{
	const cpgWorld &W = s.world[w];
	const cpgTree &T = s.tree[w];
	SapCtx c; c.keys = s.sortKA; c.vals = s.sortVA; c.rkeys = s.rkeys; c.sbb = (const longlong4_32a *)s.sapBB; c.n = W.ndynShapes;
	int lane = threadIdx.x & 31;
	int nwarps = (gridDim.x*blockDim.x) >> 5;
	for(int i = (blockIdx.x*blockDim.x + threadIdx.x) >> 5; i < c.n; i += nwarps){
		unsigned cnt = 0;
		if(lane == 0) sap_static(s, W, T, c, i, [&](int, int){ cnt++; });
		int sa = c.vals[i];
		KBB ba = gshape_kbb(s, W.shapeOff + sa);
		sap_sweep_warp(c, i, ba, sa, [&](int, int total, bool, int, int){ cnt += (lane == 0) ? total : 0; });
		if(lane == 0) s.sapCount[i] = cnt;
	}
	if(blockIdx.x == 0 && threadIdx.x == 0) s.sapCount[c.n] = 0;
}

__global__ void k_sap_emit(cpgSet s, int w)
{
	const cpgWorld &W = s.world[w];
	cpgTree &T = s.tree[w];
	SapCtx c; c.keys = s.sortKA; c.vals = s.sortVA; c.rkeys = s.rkeys; c.sbb = (const longlong4_32a *)s.sapBB; c.n = W.ndynShapes;
	unsigned total = s.sapCount[c.n];
	if(blockIdx.x == 0 && threadIdx.x == 0){
		if(total > (unsigned)W.candCap){ T.error |= CPG_ERR_CANDS; T.ncand = W.candCap; }
		else T.ncand = (int)total;
		T.narb = 0;   /* the unordered compaction counts from zero */
	}
	int lane = threadIdx.x & 31;
	int nwarps = (gridDim.x*blockDim.x) >> 5;
	for(int i = (blockIdx.x*blockDim.x + threadIdx.x) >> 5; i < c.n; i += nwarps){
		unsigned pos = s.sapCount[i];
		auto put = [&](unsigned p, int a, int b){
			if(p < (unsigned)W.candCap){
				cpgCand cd;
				cd.a = a < b ? a : b; cd.b = a < b ? b : a; cd.pair = -1;
				int slot = arb_find(s, arb_key(w, cd.a, cd.b));
				cd.idIn = (slot >= 0) ? s.arbs[slot].gjk : 0u;
				s.cands[W.candOff + p] = cd;
			}
		};
		if(lane == 0) sap_static(s, W, s.tree[w], c, i, [&](int a, int b){ put(pos, a, b); pos++; });
		pos = __shfl_sync(0xffffffffu, pos, 0);
		int sa = c.vals[i];
		KBB ba = gshape_kbb(s, W.shapeOff + sa);
		sap_sweep_warp(c, i, ba, sa, [&](int rank, int tot, bool hit, int a, int b){
			if(hit) put(pos + rank, a, b);
			pos += tot;
		});
	}
}

__device__ __forceinline__ unsigned long long unit_priority(int key)
{
	return (mix64((unsigned long long)key + 0x9e3779b97f4a7c15ull) & 0x00ffffff00000000ull) | (unsigned)key;
}

#define CPG_COLOR_ROUNDS 128
/* every this many steps all units are coloured afresh */
#define CPG_RECOLOR_PERIOD 64
/* passes that try to empty the highest colour */
#define CPG_COLOR_SQUEEZE 4

/* Colour tag kept in an arbiter's or joint's colorTag word: valid bit, the low
 * 23 bits of the stamp of the step that coloured it, the colour (< 64). */
__device__ __forceinline__ unsigned color_tag(unsigned stamp, int c)
{
	return 0x80000000u | ((stamp & 0x7FFFFFu) << 8) | (unsigned)c;
}

__device__ __forceinline__ int *unit_pad(const cpgSet &s, const cpgWorld &W, int narb, int u)
{
	return (u < narb) ? &s.arbs[s.arbList[W.candOff + u]].colorTag : &s.joints[W.consOff + (u - narb)].colorTag;
}

/* Units that were units of the previous step keep their colour (a subset
 * of a proper colouring is proper); the others are coloured by
 * Jones-Plassmann rounds with hashed priorities, each taking the lowest
 * colour free on both of its bodies.  Every CPG_RECOLOR_PERIOD steps all
 * units are coloured afresh, which bounds the drift of the colour count.
 * Then a counting sort of units by colour (empty colours dropped), with
 * per-block histograms so that each colour's counter takes one atomic per
 * block. */
__global__ void k_color_coop(cpgSet s, int w)
{
	cg::grid_group grid = cg::this_grid();
	__shared__ unsigned shHist[256], shBase[256];
	const cpgParams &P = s.params[w];
	const cpgWorld &W = s.world[w];
	cpgTree &T = s.tree[w];
	int n = T.nunits, nb = W.nbodies, narb = T.narb;
	int gtid = threadIdx.x*gridDim.x + blockIdx.x, gsz = gridDim.x*blockDim.x;
	if(n > W.unitCap){
		/* no colouring, so no per-body unit table this step */
		if(gtid == 0) s.colorCursor[13] = 1;
		return;
	}
	const int *ua = s.unitA + W.unitOff, *ub = s.unitB + W.unitOff;
	const int *ukey = s.unitKey + W.unitOff;
	int *color = s.unitLevel + W.unitOff;
	unsigned long long *claim = s.claim + W.bodyOff, *cmask = s.cmask + W.bodyOff;
	int *counter = s.colorCursor;   /* [0],[1]: remaining units per round parity */
	bool reuse = (P.stamp % CPG_RECOLOR_PERIOD) != 0;
	unsigned prevTag = color_tag(P.stamp - 1u, 0);
	for(int b = gtid; b < nb; b += gsz){ cmask[b] = 0ull; claim[b] = ~0ull; }
	if(gtid == 0){ counter[0] = 0; counter[1] = 0; counter[4] = -1; counter[5] = 0; counter[6] = -1; counter[7] = 0; counter[12] = 0; counter[13] = 0; }
	grid.sync();
	for(int u = gtid; u < n; u += gsz){
		int c = -1;
		if(reuse){
			unsigned tag = (unsigned)*unit_pad(s, W, narb, u);
			if((tag & 0xFFFFFF00u) == prevTag) c = (int)(tag & 0xFFu);
		}
		color[u] = c;
		if(c >= 0){
			/* kept units on one body have distinct colours */
			if(ua[u] >= 0) atomicOr(&cmask[ua[u]], 1ull << c);
			if(ub[u] >= 0) atomicOr(&cmask[ub[u]], 1ull << c);
		}
	}
	grid.sync();
	for(int round = 0; round < CPG_COLOR_ROUNDS; round++){
		/* claims carry the round in their top byte, newer rounds smaller,
		 * so stale claims never need clearing */
		unsigned long long tag = (unsigned long long)(255 - round) << 56;
		for(int u = gtid; u < n; u += gsz){
			if(color[u] >= 0) continue;
			unsigned long long p = tag | unit_priority(ukey[u]);
			int a = ua[u], b = ub[u];
			if(a >= 0) atomicMin(&claim[a], p);
			if(b >= 0) atomicMin(&claim[b], p);
		}
		grid.sync();
		int remaining = 0;
		for(int u = gtid; u < n; u += gsz){
			if(color[u] >= 0) continue;
			unsigned long long p = tag | unit_priority(ukey[u]);
			int a = ua[u], b = ub[u];
			if((a < 0 || __ldcg(&claim[a]) == p) && (b < 0 || __ldcg(&claim[b]) == p)){
				unsigned long long m = (a >= 0 ? __ldcg(&cmask[a]) : 0ull) | (b >= 0 ? __ldcg(&cmask[b]) : 0ull);
				int c = (m == ~0ull) ? 64 + round : __ffsll((long long)~m) - 1;
				color[u] = c;
				if(c < 64){
					/* units selected in one round share no body */
					if(a >= 0) cmask[a] = __ldcg(&cmask[a]) | (1ull << c);
					if(b >= 0) cmask[b] = __ldcg(&cmask[b]) | (1ull << c);
				}
			} else {
				remaining++;
			}
		}
		remaining = __reduce_add_sync(0xffffffffu, remaining);
		if((threadIdx.x & 31) == 0 && remaining) atomicAdd(&counter[round & 1], remaining);
		if(gtid == 0) counter[(round + 1) & 1] = 0;
		grid.sync();
		if(__ldcg(&counter[round & 1]) == 0) break;
	}
	/* fewer colours, so fewer levels: every unit of the highest colour moves
	 * to the lowest colour free on both of its bodies.  Units of one colour
	 * share no body, so they move at once without conflicts and the
	 * colouring stays proper; the passes go on while the highest colour
	 * empties (the counters alternate between two pairs of slots, one
	 * reset while the other is in use).  A colouring of units that conflict
	 * through a shared body is an edge colouring of the body graph, so it
	 * needs at least the most units on one body; on dense piles the greedy
	 * colouring is already there and nothing moves. */
	int lane = threadIdx.x & 31;
	/* only when every unit was coloured afresh: kept colours keep the
	 * result of the last squeeze */
	for(int pass = 0; pass < (reuse ? 0 : CPG_COLOR_SQUEEZE); pass++){
		int slot = 4 + 2*(pass & 1);
		int mx = -1;
		for(int u = gtid; u < n; u += gsz){ int c = color[u]; if(c < 64 && c > mx) mx = c; }
		mx = __reduce_max_sync(0xffffffffu, mx);
		if(lane == 0 && mx >= 0) atomicMax(&counter[slot], mx);
		if(gtid == 0){ counter[slot ^ 2] = -1; counter[(slot ^ 2) + 1] = 0; }
		grid.sync();
		int top = __ldcg(&counter[slot]);
		if(top <= 0) break;
		unsigned long long lower = (1ull << top) - 1ull, topBit = 1ull << top;
		int stuck = 0;
		for(int u = gtid; u < n; u += gsz){
			if(color[u] != top) continue;
			int a = ua[u], b = ub[u];
			unsigned long long m = (a >= 0 ? __ldcg(&cmask[a]) : 0ull) | (b >= 0 ? __ldcg(&cmask[b]) : 0ull);
			unsigned long long fr = ~m & lower;
			if(fr){
				int c = __ffsll((long long)fr) - 1;
				color[u] = c;
				if(a >= 0) cmask[a] = (__ldcg(&cmask[a]) & ~topBit) | (1ull << c);
				if(b >= 0) cmask[b] = (__ldcg(&cmask[b]) & ~topBit) | (1ull << c);
			} else {
				stuck++;
			}
		}
		stuck = __reduce_add_sync(0xffffffffu, stuck);
		if(lane == 0 && stuck) atomicAdd(&counter[slot + 1], stuck);
		grid.sync();
		if(__ldcg(&counter[slot + 1]) > 0) break;
	}
	/* counting sort by colour: colours past 63 come only from exhausted
	 * masks (64 + round), 255 marks a unit the rounds left uncoloured */
	for(int c = threadIdx.x; c < 256; c += blockDim.x) shHist[c] = 0u;
	__syncthreads();
	for(int u = gtid; u < n; u += gsz){
		int c = color[u];
		if(c < 0 || c > 255){ c = 255; atomicOr(&T.error, CPG_ERR_LEVELS); }
		atomicAdd(&shHist[c], 1u);
	}
	__syncthreads();
	unsigned *gHist = (unsigned *)s.colorCursor + 256;   /* [256] colour counts */
	if(blockIdx.x == 0) for(int c = threadIdx.x; c < 256; c += blockDim.x) gHist[c] = 0u;
	grid.sync();
	for(int c = threadIdx.x; c < 256; c += blockDim.x)
		shBase[c] = shHist[c] ? atomicAdd(&gHist[c], shHist[c]) : 0u;
	grid.sync();
	/* levels over the non-empty colours; every block derives the same
	 * offsets from the counts */
	int *start = s.levelStart + W.unitOff + w;
	__shared__ int shLevel[256], shStart[256], shN;
	if(threadIdx.x == 0){
		int lev = 0, acc = 0;
		for(int c = 0; c < 256; c++){
			unsigned cnt = __ldcg(&gHist[c]);
			if(cnt){ shLevel[c] = lev; shStart[c] = acc; acc += (int)cnt; lev++; }
			else shLevel[c] = -1;
		}
		shN = lev;
	}
	__syncthreads();
	int nlev = shN;
	if(blockIdx.x == 0){
		for(int c = threadIdx.x; c < 256; c += blockDim.x)
			if(shLevel[c] >= 0) start[shLevel[c]] = shStart[c];
		if(threadIdx.x == 0){
			start[nlev] = n;
			T.nlevels = nlev;
			if(nlev > T.maxChain) T.maxChain = nlev;
		}
	}
	for(int c = threadIdx.x; c < 256; c += blockDim.x) shHist[c] = 0u;
	__syncthreads();
	int *order = s.unitOrder + W.unitOff;
	unsigned newTagBase = color_tag(P.stamp, 0);
	/* the per-body unit table serves the dataflow sweep and the per-body
	 * warm start (which also counts as the sweep's pass 0 done) */
	bool flow = s.flowSolve != 0, table = flow || s.warmGather;
	int *fpos = s.flowPos + 64*(size_t)W.bodyOff;
	for(int u = gtid; u < n; u += gsz){
		int c = color[u];
		if(c < 0 || c > 255) c = 255;
		int pos = shStart[c] + shBase[c] + atomicAdd(&shHist[c], 1u);
		order[pos] = u;
		*unit_pad(s, W, narb, u) = (int)(c < 64 ? (newTagBase | (unsigned)c) : 0u);
		if(table){
			if(flow) s.flowDone[W.unitOff + u] = s.warmGather ? 1 : 0;
			if(c < 64){
				if(ua[u] >= 0) fpos[64*ua[u] + c] = pos;
				if(ub[u] >= 0) fpos[64*ub[u] + c] = pos;
			} else {
				counter[13] = 1;
			}
		}
	}
	if(!flow) return;
	grid.sync();
	if(__ldcg(&counter[13])) return;
	/* predecessors of the dataflow sweep: on each body, the unit of the
	 * next lower colour in the same pass, or, for the body's lowest colour,
	 * the unit of its highest colour in the previous pass (none when that
	 * is the unit itself) */
	int *pred = s.flowPred + 2*(size_t)W.unitOff;
	for(int k = gtid; k < n; k += gsz){
		int u = __ldcg(&order[k]);
		int c = __ldcg(&color[u]);
#pragma unroll
		for(int side = 0; side < 2; side++){
			int x = side ? ub[u] : ua[u];
			int pr = -1;
			if(x >= 0){
				unsigned long long m = __ldcg(&cmask[x]);
				unsigned long long lower = m & ((1ull << c) - 1ull);
				if(lower){
					pr = __ldcg(&fpos[64*x + 63 - __clzll((long long)lower)]) << 1;
				} else {
					int q = __ldcg(&fpos[64*x + 63 - __clzll((long long)m)]);
					pr = (q == k) ? -1 : ((q << 1) | 1);
				}
			}
			pred[2*k + side] = pr;
		}
	}
}

/* 96 quads per block: the quad-lane solve holds its next row in registers
 * (about 170 per thread, so 384 threads fill the register file) */
#define CPG_COOP_SOLVE_THREADS 256

/* Whether a level of U units, dealt round-robin over `blocks` blocks of
 * the whole-grid solve, takes fewer FP64 instructions on the busiest
 * sub-partition on two lanes per contact (~33 per lane fused, ~50 exact)
 * than on four (~25, ~37): a block's warps go round-robin to its four
 * sub-partitions. */
template<bool FUSED>
__device__ __forceinline__ bool coop_two_lanes(int U, int blocks)
{
	int ub = (U + blocks - 1)/blocks;
	int w4 = (4*ub + 31) >> 5, w2 = (2*ub + 31) >> 5;
	return ((w2 + 3) >> 2)*(FUSED ? 33 : 50) < ((w4 + 3) >> 2)*(FUSED ? 25 : 37);
}

/* ---- dataflow sweep (coloured mode) ----
 * Instead of a grid barrier after every colour, each unit waits for the
 * units before it in the sweep on its two bodies (flowPred, from the
 * colouring) and then marks its pass done (flowDone = pass + 1).  Every
 * body still sees its updates in the same order, so the results are the
 * barrier sweep's bit for bit.  Warps take their units in (pass, colour)
 * order and wait only for smaller ones, and a cooperative launch keeps
 * every block resident, so the waits always end; they are bounded all the
 * same: past CPG_FLOW_SPIN polls the sweep latches CPG_ERR_FLOW, raises
 * the abort word and stops waiting.  A warp waits for all of its units
 * together, so its lanes stay converged for the FP64 work.
 * Measured on 20,000 settled circles it is slower than the barrier sweep
 * (0.77 against 0.51 ms): the longest chain of dependent units still
 * crosses every colour of every pass, and each link pays a release, a
 * poll and the body loads, more than one grid barrier per colour costs.
 * It is kept as an option (cpGpuDebugSetFlowSolve). */
#define CPG_FLOW_SPIN (1 << 20)

__device__ __forceinline__ int ld_acquire_gpu(const int *p)
{
	int v;
	asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}

__device__ __forceinline__ void st_release_gpu(int *p, int v)
{
	asm volatile("st.release.gpu.global.b32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

/* Whole warp: wait until the predecessors of this lane's unit k (or none,
 * k < 0) have finished the passes this one needs. */
__device__ __forceinline__ void flow_wait(const int *pred, const int *done, int *abortWord, int *err, int k, int pass, int limit)
{
	int f0 = -1, t0 = 0, f1 = -1, t1 = 0;
	if(k >= 0){
		int p0 = pred[2*k], p1 = pred[2*k + 1];
		if(p0 >= 0){ t0 = pass + ((p0 & 1) ? 0 : 1); if(t0 > 0) f0 = p0 >> 1; }
		if(p1 >= 0){ t1 = pass + ((p1 & 1) ? 0 : 1); if(t1 > 0) f1 = p1 >> 1; }
	}
	bool ready = false;
	for(int it = 0;; it++){
		if(!ready) ready = (f0 < 0 || ld_acquire_gpu(done + f0) >= t0) && (f1 < 0 || ld_acquire_gpu(done + f1) >= t1);
		if(__all_sync(0xffffffffu, ready)) return;
		if((it & 31) == 31){
			if(__any_sync(0xffffffffu, ld_acquire_gpu(abortWord) != 0)) return;
			if(it >= limit){
				if((threadIdx.x & 31) == 0){ atomicOr(err, CPG_ERR_FLOW); atomicExch(abortWord, 1); }
				return;
			}
		}
	}
}

/* Whole warp: this lane's unit k (leader lanes only) has finished `pass`;
 * every lane's body and row stores are made visible first. */
__device__ __forceinline__ void flow_done(int *done, int k, int pass, bool leader)
{
	asm volatile("fence.acq_rel.gpu;" ::: "memory");
	__syncwarp();
	if(leader && k >= 0) st_release_gpu(done + k, pass + 1);
}

/* Levels (ordered mode) or colours (coloured mode) of one large world,
 * with the whole grid: grid.sync() between levels, or, in the coloured
 * mode, the dataflow waits above.  Packed body state is read past the L1
 * (__ldcg), since other blocks write it; a row is always handled by the
 * same lanes, in one SM, so its own accumulator updates are coherent.
 * Each warp walks a level's units in warp-uniform steps, so that the
 * dataflow waits are whole-warp. */
template<bool FUSED>
__global__ void __launch_bounds__(CPG_COOP_SOLVE_THREADS, 1) k_solve_coop(cpgSet s, int w)
{
	cg::grid_group grid = cg::this_grid();
	const cpgParams &P = s.params[w];
	const cpgWorld &W = s.world[w];
	cpgTree &T = s.tree[w];
	int nunits = T.nunits, nlev = T.nlevels;
	if(nunits > W.unitCap || nlev < 1) return;
	const int *start = s.levelStart + W.unitOff + w;
	cpgRow *rows = s.rows + W.unitOff;
	double *bodies = s.pbody + 8*(size_t)W.bodyOff;
	int iters = P.iterations;
	double dt_coef = P.dt_coef, dt = P.dt;
	bool flow = FUSED && s.flowSolve && s.colorCursor[13] == 0;
	/* the waits' poll limit, and (a test of the limit) completions that
	 * are never published, so that every wait with a predecessor runs out */
	int flowLimit = s.flowSpin > 0 ? s.flowSpin : CPG_FLOW_SPIN;
	bool publish = !s.flowWithhold;
	/* coloured mode: k_integrate_vel has applied the cached impulses */
	int pass0 = (FUSED && s.warmGather && s.colorCursor[13] == 0) ? 1 : 0;
	const int *pred = s.flowPred + 2*(size_t)W.unitOff;
	int *done = s.flowDone + W.unitOff;
	int *abortWord = s.colorCursor + 12;
	/* four lanes per unit; a level's units are dealt round-robin over the
	 * blocks (unit i to block i % gridDim.x), so that every SM's FP64 pipes
	 * take a share of each level */
	int lane4 = threadIdx.x & 3;
	int quad = (threadIdx.x >> 2)*gridDim.x + blockIdx.x, nq = (gridDim.x*blockDim.x) >> 2;
	unsigned qmask = 0xFu << (threadIdx.x & 28);
	/* the quad's first unit of the next level is read before the barrier,
	 * so that only the body loads remain after it */
	/* a level whose units fill more than one warp per sub-partition on four
	 * lanes runs on two (one lane per part, both bodies): half the warps,
	 * each with ~1.3x the instructions */
	int pair = (threadIdx.x >> 1)*gridDim.x + blockIdx.x, np2 = (gridDim.x*blockDim.x) >> 1;
	bool bias = (threadIdx.x & 1) != 0;
	/* exact order: a level no wider than one block's quads runs on block 0
	 * alone, and a run of such levels needs a grid barrier only after its
	 * last level (a block barrier between its levels, the next level's row
	 * read before it).  A level's units share no body, so which quads
	 * apply them changes no result. */
	const int narrowMax = FUSED ? 0 : (blockDim.x >> 2);
	QuadRow qn;
	bool haveN = false;
	QuadRow q;
	int k = start[0] + quad;
	bool two = coop_two_lanes<FUSED>(start[1] - start[0], gridDim.x);
	bool have = !two && k < start[1] && (FUSED || (start[1] - start[0]) > narrowMax);
	if(have) quad_load(q, rows[k], lane4);
	for(int pass = pass0; pass <= iters; pass++){
		for(int l = 0; l < nlev; l++){
			int e = start[l + 1];
			bool narrow = !FUSED && (e - start[l]) <= narrowMax;
			if(narrow){
				if(blockIdx.x == 0){
					int k2 = start[l] + (threadIdx.x >> 2);
					if(k2 < e){
						if(!haveN) quad_load(qn, rows[k2], lane4);
						if(qn.kind == 0) quad_apply<true, FUSED>(qn, rows + k2, bodies, pass, dt_coef, qmask, lane4);
						else if(lane4 == 0) solve_row<true>(rows, k2, bodies, pass, dt_coef, dt);
					}
					/* the next narrow level's row, before the block barrier
					 * (a single level re-reads the row this quad wrote) */
					int nl2 = l + 1, np2 = pass;
					if(nl2 == nlev){ nl2 = 0; np2++; }
					int kq = start[nl2] + (threadIdx.x >> 2);
					haveN = np2 <= iters && (start[nl2 + 1] - start[nl2]) <= narrowMax && kq < start[nl2 + 1];
					__syncwarp(qmask);
					if(haveN) quad_load(qn, rows[kq], lane4);
					__syncthreads();
				}
			} else if(two){
				for(int k2 = start[l] + pair; __any_sync(0xffffffffu, k2 < e); k2 += np2){
					bool has = k2 < e;
					PairRow pr;
					if(has) pair_load(pr, rows[k2], bias);
					if(flow) flow_wait(pred, done, abortWord, &T.error, has ? k2 : -1, pass, flowLimit);
					if(has){
						if(pr.kind == 0) pair_apply<true, FUSED>(pr, rows + k2, bodies, pass, dt_coef, bias);
						else if(!bias) solve_row<true>(rows, k2, bodies, pass, dt_coef, dt);
					}
					if(flow) flow_done(done, has ? k2 : -1, pass, !bias && publish);
				}
			} else {
				/* levels wider than the grid take several rounds */
				for(int k2 = k; __any_sync(0xffffffffu, k2 < e); k2 += nq){
					bool has = k2 < e;
					if(has && k2 != k) quad_load(q, rows[k2], lane4);
					if(flow) flow_wait(pred, done, abortWord, &T.error, has ? k2 : -1, pass, flowLimit);
					if(has){
						if(q.kind == 0) quad_apply<true, FUSED>(q, rows + k2, bodies, pass, dt_coef, qmask, lane4);
						else if(lane4 == 0) solve_row<true>(rows, k2, bodies, pass, dt_coef, dt);
					}
					if(flow) flow_done(done, has ? k2 : -1, pass, lane4 == 0 && publish);
				}
			}
			int nl = l + 1, npass = pass;
			if(nl == nlev){ nl = 0; npass++; }
			bool nextNarrow = !FUSED && npass <= iters && (start[nl + 1] - start[nl]) <= narrowMax;
			if(narrow && nextNarrow) continue;
			k = start[nl] + quad;
			two = coop_two_lanes<FUSED>(start[nl + 1] - start[nl], gridDim.x);
			have = !two && !nextNarrow && npass <= iters && k < start[nl + 1];
			if(flow){
				/* the warp synchronised after its last unit, so a row this
				 * quad just wrote (a single level) reads back current */
				if(have) quad_load(q, rows[k], lane4);
			} else {
				/* with a single level the next row is the one just written
				 * by lanes 0 and 2 of this quad */
				__syncthreads();
				if(have) quad_load(q, rows[k], lane4);
				grid.sync();
			}
		}
	}
}

/* ------------------------------------------------------------------ */
/* Launchers */

static inline int blocks_for(int n, int bs) { return (n + bs - 1)/bs > 0 ? (n + bs - 1)/bs : 1; }

static cudaError_t check_launch(const char *what)
{
	cudaError_t e = cudaGetLastError();
	if(e != cudaSuccess) fprintf(stderr, "chipmunk_gb300: launch of %s failed: %s\n", what, cudaGetErrorString(e));
	return e;
}

extern "C" int cpg_launch_sleep_edits(const cpgSet *s, const unsigned long long *keys, const int *ops, const unsigned *stamps, int n,
                                      const unsigned long long *listKeys, int nlist, void *stream)
{
	cudaStream_t st = (cudaStream_t)stream;
	if(n > 0) LAUNCH(k_sleep_flags<<<1, 1, 0, st>>>(*s, keys, ops, stamps, n));
	if(nlist >= 0) LAUNCH(k_set_list<<<1, 1024, 0, st>>>(*s, listKeys, nlist));
	return check_launch("k_sleep_edits") == cudaSuccess ? 0 : -1;
}

extern "C" int cpg_launch_gather_slots(const cpgSet *s, const int *slots, cpgArb *out, int n, void *stream)
{
	if(n <= 0) return 0;
	LAUNCH(k_gather_slots<<<blocks_for(n, 128), 128, 0, (cudaStream_t)stream>>>(*s, slots, out, n));
	return check_launch("k_gather_slots") == cudaSuccess ? 0 : -1;
}

extern "C" int cpg_launch_put_arbs(const cpgSet *s, const int *slots, const cpgArb *recs, int n, void *stream)
{
	if(n <= 0) return 0;
	LAUNCH(k_put_arbs<<<blocks_for(n, 128), 128, 0, (cudaStream_t)stream>>>(*s, slots, recs, n));
	return check_launch("k_put_arbs") == cudaSuccess ? 0 : -1;
}

extern "C" int cpg_launch_shape_arbs(const cpgSet *s, int shape, int *slots, int *count, int cap, void *stream)
{
	cudaStream_t st = (cudaStream_t)stream;
	cudaMemsetAsync(count, 0, sizeof(int), st);
	LAUNCH(k_shape_arbs<<<blocks_for(s->arbCap, 256), 256, 0, st>>>(*s, shape, slots, count, cap));
	return check_launch("k_shape_arbs") == cudaSuccess ? 0 : -1;
}

extern "C" int cpg_launch_gather_pairs(const cpgSet *s, int world, int *out, int n, void *stream)
{
	if(n <= 0) return 0;
	LAUNCH(k_gather_pairs<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(*s, world, (int2 *)out, n));
	return check_launch("k_gather_pairs") == cudaSuccess ? 0 : -1;
}

extern "C" int cpg_launch_gather_keys(const cpgSet *s, const unsigned long long *keys, cpgArb *out, int n, void *stream)
{
	if(n <= 0) return 0;
	LAUNCH(k_gather_keys<<<blocks_for(n, 128), 128, 0, (cudaStream_t)stream>>>(*s, keys, out, n));
	return check_launch("k_gather_keys") == cudaSuccess ? 0 : -1;
}

extern "C" int cpg_launch_gather_arbs(const cpgSet *s, int world, cpgArb *out, int n, void *stream)
{
	LAUNCH(k_gather_arbs<<<blocks_for(n, 128), 128, 0, (cudaStream_t)stream>>>(*s, world, out, n));
	return check_launch("k_gather_arbs") == cudaSuccess ? 0 : -1;
}

extern "C" int cpg_launch_body_states(const cpgSet *s, int w, double *out, int n, void *stream)
{
	if(n <= 0) return 0;
	LAUNCH(k_body_states<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(*s, w, out, n));
	return check_launch("k_body_states") == cudaSuccess ? 0 : -1;
}

extern "C" int cpg_launch_apply_ops(const cpgSet *s, void *stream)
{
	cudaStream_t st = (cudaStream_t)stream;
	LAUNCH(k_apply_ops<<<blocks_for(s->nworlds, 64), 64, 0, st>>>(*s));
	return check_launch("k_apply_ops") == cudaSuccess ? 0 : -1;
}

extern "C" int cpg_launch_transfer(const cpgSet *to, const cpgSet *from, const int *bodyMap, const unsigned char *deadShape,
                                   int *slotMap, void *stream)
{
	cudaStream_t st = (cudaStream_t)stream;
	LAUNCH(k_transfer_pools<<<152*2, 256, 0, st>>>(*to, *from));
	LAUNCH(k_transfer_arbs<<<blocks_for(from->arbCap, 256), 256, 0, st>>>(*to, *from, bodyMap, deadShape, slotMap));
	LAUNCH(k_transfer_list<<<1, 32, 0, st>>>(*to, *from, slotMap));
	return check_launch("k_transfer") == cudaSuccess ? 0 : -1;
}

static int coop_blocks(const void *kernel, int threads)
{
	static int sms = 0;
	if(!sms){ int dev = 0; cudaGetDevice(&dev); cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev); }
	int per = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0);
	if(per < 1) per = 1;
	return sms*per;
}

static cudaError_t launch_coop(const void *kernel, int threads, cpgSet *s, int w, cudaStream_t st)
{
	/* one block per SM: the fewer blocks a grid barrier waits for, the
	 * cheaper it is, and a colour rarely has more units than threads */
	static const void *kernels[8];
	static int blocks[8];
	int slot = 0;
	while(slot < 8 && kernels[slot] && kernels[slot] != kernel) slot++;
	if(slot == 8) return cudaErrorInvalidValue;
	kernels[slot] = kernel;
	int *cache = &blocks[slot];
	if(!*cache){
		int most = coop_blocks(kernel, threads);
		int sms = 0, dev = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		*cache = most < sms ? most : sms;
	}
	void *args[] = { (void *)s, (void *)&w };
	g_launches++;
	int nb = *cache;
	if(s->hostCoopBlocks > 0 && s->hostCoopBlocks < nb) nb = s->hostCoopBlocks;
	return cudaLaunchCooperativeKernel(kernel, dim3(nb), dim3(threads), args, 0, st);
}

/* Single-world sets with at least this many solver units use the
 * cooperative whole-grid solve; smaller ones keep one block. */
#define CPG_COOP_UNITS 2048
/* Worlds up to this many bodies keep their solver body state in shared
 * memory (64 bytes each, 200 KB at most). */
#define CPG_STAGED_BODIES 3200
/* Worlds whose tree node pool has at most this many nodes run the tree step
 * with the pool in shared memory (64 bytes a node, 192 KB at most). */
#define CPG_STAGED_NODES 2048

/* `h` is the host copy of the set's sizes (same struct, host values). */
/* A many-world step as a CUDA graph: captured from cpg_launch_step, and
 * captured again when the launch arguments (the set as the host holds it,
 * the mode) change. */
struct cpgStepGraph {
	cudaGraphExec_t exec;
	cpgSet key;
	int mode;
	long long launches;
	int valid;
};

extern "C" void cpg_step_graph_free(void *cache)
{
	cpgStepGraph *g = (cpgStepGraph *)cache;
	if(!g) return;
	if(g->valid) cudaGraphExecDestroy(g->exec);
	free(g);
}

extern "C" int cpg_launch_step_part(const cpgSet *s, const cpgSet *h, int mode, void *stream, float *phase_ms, int part);
extern "C" int cpg_launch_step(const cpgSet *s, const cpgSet *h, int mode, void *stream, float *phase_ms)
{
	return cpg_launch_step_part(s, h, mode, stream, phase_ms, 0);
}

extern "C" int cpg_launch_step_graph(const cpgSet *s, int mode, void *stream, void **cache)
{
	cudaStream_t st = (cudaStream_t)stream;
	cpgStepGraph *g = (cpgStepGraph *)*cache;
	if(!g){
		g = (cpgStepGraph *)calloc(1, sizeof(cpgStepGraph));
		if(!g) return cpg_launch_step(s, s, mode, stream, NULL);
		*cache = g;
	}
	if(!g->valid || g->mode != mode || memcmp(&g->key, s, sizeof(cpgSet)) != 0){
		if(g->valid){ cudaGraphExecDestroy(g->exec); g->valid = 0; }
		long long before = g_launches;
		if(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess){
			cudaGetLastError();
			return cpg_launch_step(s, s, mode, stream, NULL);
		}
		int rc = cpg_launch_step(s, s, mode, stream, NULL);
		cudaGraph_t graph = NULL;
		cudaError_t e = cudaStreamEndCapture(st, &graph);
		long long n = g_launches - before;
		g_launches = before;
		if(rc != 0 || e != cudaSuccess || !graph){
			if(graph) cudaGraphDestroy(graph);
			cudaGetLastError();
			return cpg_launch_step(s, s, mode, stream, NULL);
		}
		e = cudaGraphInstantiate(&g->exec, graph, 0);
		cudaGraphDestroy(graph);
		if(e != cudaSuccess){
			cudaGetLastError();
			return cpg_launch_step(s, s, mode, stream, NULL);
		}
		g->key = *s; g->mode = mode; g->launches = n; g->valid = 1;
	}
	if(cudaGraphLaunch(g->exec, st) != cudaSuccess) return -1;
	g_launches += g->launches;
	return 0;
}

extern "C" int cpg_launch_replay_solve(const cpgSet *s, const cpgAdj *a, int nsteps, void *stream)
{
	cudaStream_t st = (cudaStream_t)stream;
	int stagedMax = s->hostMaxBodies <= CPG_STAGED_BODIES ? s->hostMaxBodies : 0;
	size_t smem = (size_t)stagedMax*8*sizeof(double);
	static size_t smemSet = 0;
	if(smem > 48*1024 && smem > smemSet){
		cudaFuncSetAttribute(k_replay_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		smemSet = smem;
	}
	/* the forward's (tuned) solve block size */
	int threads = s->hostSolveThreads > 0 ? s->hostSolveThreads : (s->nworlds*nsteps >= 152 ? 128 : 256);
	LAUNCH(k_replay_solve<<<dim3(s->nworlds, nsteps), threads, smem, st>>>(*s, *a, stagedMax));
	return check_launch("k_replay_solve") == cudaSuccess ? 0 : -1;
}

/* part 0: the whole step; part 1: up to the arbiter list (cpSpaceStep.c
 * up to :372); part 2: the rest, from the cache filter on (:378-445);
 * parts 3 and 4 split part 2 after the filter.  Between the parts the host
 * runs cpSpaceProcessComponents and the collision-handler callbacks. */
extern "C" int cpg_launch_step_part(const cpgSet *s, const cpgSet *h, int mode, void *stream, float *phase_ms, int part)
{
	cudaStream_t st = (cudaStream_t)stream;
	if(part != 0) phase_ms = NULL;
	int W = h->nworlds;
	cudaEvent_t ev[8];
	bool timing = (phase_ms != NULL);
	if(timing){
		for(int i = 0; i < 8; i++) cudaEventCreate(&ev[i]);
		cudaEventRecord(ev[0], st);
	}
	/* grid.x for per-world candidate/unit kernels: one world spans many
	 * blocks; many worlds get one block row each */
	int perWorldX = (W == 1) ? 152*4 : 1;
	bool colored = (mode == 1 && W == 1);
	cpgSet sv = *s;
	/* the per-body warm start needs the colouring's per-body unit table */
	sv.warmGather = (colored && !h->tape.on && s->warmGather) ? 1 : 0;
	sv.parMark = (!colored && W == 1 && s->parMark) ? 1 : 0;

	/* a refused cooperative launch (occupancy, an unsupported context)
	 * fails the step: the kernels after it would run on a half-done step */
	cudaError_t coop = cudaSuccess;
#define COOP(kernel, threads) do { cudaError_t e_ = launch_coop((const void *)(kernel), (threads), &sv, 0, st); if(e_ != cudaSuccess && coop == cudaSuccess) coop = e_; } while(0)
	if(part == 8) goto after_position;
	if(part >= 2 && part != 7) goto second;
	cudaMemsetAsync(s->stats, 0, 16*sizeof(int), st);
	LAUNCH(k_reset_prev<<<dim3(perWorldX, W), 128, 0, st>>>(*s));
	LAUNCH(k_integrate_pos<<<blocks_for(h->totalBodies, 128), 128, 0, st>>>(*s));
	if(part == 7) goto done;
after_position:
	LAUNCH(k_shape_cache<<<blocks_for(h->totalShapes, 128), 128, 0, st>>>(*s));
	if(timing) cudaEventRecord(ev[1], st);
	if(colored){
		int n = h->hostNdyn;
		COOP(k_sap_sort, SAP_THREADS);
		LAUNCH(k_sap_count<<<blocks_for(32*n, 256), 256, 0, st>>>(*s, 0));
		LAUNCH(k_scan_excl<<<1, 1024, 0, st>>>(s->sapCount, n + 1, NULL));
		LAUNCH(k_sap_emit<<<blocks_for(32*n, 256), 256, 0, st>>>(*s, 0));
	} else {
		/* node pools of up to CPG_STAGED_NODES nodes (96 B each) run from
		 * shared memory; larger worlds use the global pool */
		int staged = h->hostMaxNodes <= CPG_STAGED_NODES ? h->hostMaxNodes : 0;
		/* the tree is one serial thread per world: many worlds gain more
		 * from residency (a pool sized for the largest world would hold
		 * every block's shared memory) than from shared-memory latency */
		if(h->hostTreeStage >= 0){ if(h->hostTreeStage < staged) staged = h->hostTreeStage; }
		else if(W > 2*152 && staged > 384) staged = 0;
		size_t smem = (size_t)staged*sizeof(cpgNode);
		static size_t treeSmemSet = 0;
		if(smem > 48*1024 && smem > treeSmemSet){
			cudaFuncSetAttribute(k_tree, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
			treeSmemSet = smem;
		}
		/* one warp per world in a batch; a single world's leaf scan takes
		 * 256 threads (thread 0 alone reinserts and marks) */
		if(h->useHash){
			/* the grids (two cell arrays, two bin pools) and three ints per
			 * node in shared memory when they fit */
			size_t hbytes = sizeof(int)*(2*(size_t)h->numcells + 4*(size_t)h->gbinCap + 7*(size_t)h->totalNodes);
			int hstaged = hbytes <= 200*1024;
			static size_t hashSmemSet = 0;
			if(hstaged && hbytes > 48*1024 && hbytes > hashSmemSet){
				cudaFuncSetAttribute(k_hash_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hbytes);
				hashSmemSet = hbytes;
			}
			LAUNCH(k_hash_step<<<1, 256, hstaged ? hbytes : 0, st>>>(*s, hstaged));
		}
		else {
			LAUNCH(k_tree<<<W, W == 1 ? 256 : 32, smem, st>>>(sv, staged));
			if(sv.parMark) COOP(k_tree_mark, CPG_MARK_THREADS);
		}
	}
	if(timing) cudaEventRecord(ev[2], st);
	cudaMemsetAsync(s->nbCount, 0, CPG_PAIR_TYPES*sizeof(int), st);
	LAUNCH(k_narrow_classify<<<dim3(perWorldX, W), 128, 0, st>>>(*s));
	LAUNCH(k_narrow_collide<<<152*3, 128, 0, st>>>(*s));
	if(timing) cudaEventRecord(ev[3], st);
	LAUNCH(k_arb_update<<<dim3(perWorldX, W), 128, 0, st>>>(*s));
	if(colored){
		LAUNCH(k_solve_list_any<<<152*2, 256, 0, st>>>(*s, 0));
		LAUNCH(k_units_joints<<<blocks_for(h->totalCons > 0 ? h->totalCons : 1, 128), 128, 0, st>>>(*s, 0));
	} else {
		LAUNCH(k_solve_list<<<W, 256, 0, st>>>(*s));
	}
	if(part == 1 || part == 8) goto done;
second:
	if(part == 6) goto after_velocity;
	if(part != 4 && part != 5){
		if(s->sepCount) cudaMemsetAsync(s->sepCount, 0, sizeof(int), st);
		LAUNCH(k_arb_filter<<<blocks_for(h->arbCap, 256), 256, 0, st>>>(*s));
	}
	if(part == 3) goto done;
	if(timing) cudaEventRecord(ev[4], st);
	if(colored) COOP(k_color_coop, 512);
	else if(W == 1){
		static bool schedSmemSet = false;
		if(!schedSmemSet){
			cudaFuncSetAttribute(k_schedule_one, cudaFuncAttributeMaxDynamicSharedMemorySize, CPG_SCHED_SMEM_INTS*(int)sizeof(int));
			schedSmemSet = true;
		}
		LAUNCH(k_schedule_one<<<1, CPG_SCHED_THREADS, CPG_SCHED_SMEM_INTS*sizeof(int), st>>>(*s));
	}
	else LAUNCH(k_schedule<<<blocks_for(W, 32), 32, 0, st>>>(*s));
	if(timing) cudaEventRecord(ev[5], st);
	LAUNCH(k_build_rows<<<dim3(perWorldX, W), 128, 0, st>>>(*s));
	if(h->tape.on) cpg_launch_tape(s, st);
	LAUNCH(k_integrate_vel<<<blocks_for(h->totalBodies, 128), 128, 0, st>>>(sv));
	if(h->tape.on) cpg_launch_tape_vel(s, st);
	if(part == 5) goto done;
after_velocity:
	if(timing) cudaEventRecord(ev[6], st);
	if(W == 1 && colored){
		COOP(k_solve_coop<true>, CPG_COOP_SOLVE_THREADS);
	} else if(W == 1 && h->hostUnitsHint >= CPG_COOP_UNITS && !h->tape.on){
		COOP(k_solve_coop<false>, CPG_COOP_SOLVE_THREADS);
	} else {
		int stagedMax = h->hostMaxBodies <= CPG_STAGED_BODIES ? h->hostMaxBodies : 0;
		if(h->hostSolveStage >= 0 && h->hostSolveStage < stagedMax) stagedMax = h->hostSolveStage;
		size_t smem = (size_t)stagedMax*8*sizeof(double);
		static size_t smemSet = 0;
		if(smem > 48*1024 && smem > smemSet){
			cudaFuncSetAttribute(k_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
			smemSet = smem;
		}
		/* many worlds: small blocks keep more worlds resident (registers
		 * limit a 256-thread block to two per SM); one world: wide levels */
		int threads = h->hostSolveThreads > 0 ? h->hostSolveThreads : (W >= 152 ? 128 : 256);
		LAUNCH(k_solve<<<W, threads, smem, st>>>(*s, stagedMax));
	}
	LAUNCH(k_writeback<<<dim3(perWorldX, W), 128, 0, st>>>(*s));
	LAUNCH(k_unpack_bodies<<<blocks_for(h->totalBodies, 128), 128, 0, st>>>(*s));
	if(timing) cudaEventRecord(ev[7], st);
	LAUNCH(k_stats<<<1, 256, 0, st>>>(*s));
done:
#undef COOP
	cudaError_t e = check_launch("step");
	if(coop != cudaSuccess){
		fprintf(stderr, "chipmunk_gb300: a cooperative launch was refused: %s\n", cudaGetErrorString(coop));
		e = coop;
	}
	if(timing){
		cudaEventSynchronize(ev[7]);
		for(int i = 0; i < 7; i++) cudaEventElapsedTime(&phase_ms[i], ev[i], ev[i + 1]);
		for(int i = 0; i < 8; i++) cudaEventDestroy(ev[i]);
	}
	return e == cudaSuccess ? 0 : -1;
}

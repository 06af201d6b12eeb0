/*
 * TEST INFRASTRUCTURE — CPU oracle (see flowshop_oracle.h for the scope and
 * the reference files it restates). Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load this code.
 *
 * The bound is restated with the reference's own cost profile: every node
 * recomputes its front times, its back times (per start machine, O(b*m^2))
 * and walks all n jobs of every pair's Johnson order, as
 * src/bound_flowshop.cpp:841-895 and :64-77 do. That keeps the CPU timing
 * of this port representative of the reference CPU path.
 */
#include "flowshop_oracle.h"

#include <limits.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* Seeded instances                                                    */
/* ------------------------------------------------------------------ */

static uint64_t sm64(uint64_t *s)
{
	uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
	return z ^ (z >> 31);
}

/* Uniform integer in [0, k) by rejection (no modulo bias). */
static uint64_t sm64_below(uint64_t *s, uint64_t k)
{
	uint64_t lim = (UINT64_MAX / k) * k;
	for (;;) {
		uint64_t x = sm64(s);
		if (x < lim)
			return x % k;
	}
}

void fs_gen_instance(uint64_t seed, int n, int m, int32_t *p)
{
	uint64_t s = seed;
	for (int k = 0; k < m; k++)
		for (int j = 0; j < n; j++)
			p[k * n + j] = (int32_t)(1 + sm64_below(&s, 99));
}

/* Taillard's generator as the reference draws it
 * (src/instance_flowshop.cpp:74-89): the Lehmer step s <- 16807 s mod
 * (2^31 - 1), here by direct 64-bit arithmetic (the reference uses Schrage's
 * decomposition: same values), then a time 1 + floor(q * 99) with the
 * quotient q = s / (2^31 - 1) taken in single precision, machine-major. */
void fs_taillard_instance(int64_t seed, int n, int m, int32_t *p)
{
	int64_t s = seed;
	for (int k = 0; k < m; k++)
		for (int j = 0; j < n; j++) {
			s = (int64_t)(((uint64_t)s * 16807u) % 2147483647u);
			float q = (float)s / (float)2147483647;
			p[k * n + j] = (int32_t)(1 + (int64_t)((double)q * 99.0));
		}
}

void fs_random_pool(uint64_t seed, int n, int64_t count, double leaf_share,
                    int32_t *perms, int32_t *l1, int32_t *l2)
{
	uint64_t s = seed;
	for (int64_t r = 0; r < count; r++) {
		int32_t *pr = perms + r * n;
		for (int j = 0; j < n; j++)
			pr[j] = j;
		for (int j = n - 1; j > 0; j--) {
			int k = (int)sm64_below(&s, (uint64_t)j + 1);
			int32_t t = pr[j];
			pr[j] = pr[k];
			pr[k] = t;
		}
		double u = (double)(sm64(&s) >> 11) * (1.0 / 9007199254740992.0);
		if (u < leaf_share) {
			int b = (int)sm64_below(&s, (uint64_t)n - 1); /* 0..n-2 */
			l2[r] = n - b;
			l1[r] = n - b - 1;
		} else {
			int f = (int)sm64_below(&s, (uint64_t)n - 2);        /* 0..n-3 */
			int b = (int)sm64_below(&s, (uint64_t)(n - 2 - f)); /* 0..n-3-f */
			l1[r] = f - 1;
			l2[r] = n - b;
		}
	}
}

/* ------------------------------------------------------------------ */
/* Bound precompute (src/bound_flowshop.cpp:486-659)                   */
/* ------------------------------------------------------------------ */

struct fs_bound {
	int n, m, P;
	int32_t *p;       /* m x n */
	int32_t *mach[2]; /* P: machine pair in lexicographic order (:500-508) */
	int32_t *lag;     /* P x n: sum of p strictly between the pair (:486-498) */
	int32_t *johnson; /* P x n: Johnson-with-lags order (:627-643) */
	int32_t *min_arr; /* m: static heads (:510-538) */
	int32_t *min_dep; /* m: static tails (:510-538) */
};

/* Sort keys of the Johnson rule; `grp` is 1 (p1 < p2) or 2. */
typedef struct {
	const int32_t *grp;
	const int32_t *key;
} fs_keys;

/* estInf / estSup (src/bound_flowshop.cpp:579-595): group 1 ascending by
 * key, then group 2 descending by key. */
static int key_lt(const fs_keys *k, int i, int j)
{
	if (k->grp[i] == k->grp[j]) {
		if (k->grp[i] == 1)
			return k->key[i] < k->key[j];
		return k->key[i] > k->key[j];
	}
	return k->grp[i] < k->grp[j];
}

static int key_gt(const fs_keys *k, int i, int j)
{
	if (k->grp[i] == k->grp[j]) {
		if (k->grp[i] == 1)
			return k->key[i] > k->key[j];
		return k->key[i] < k->key[j];
	}
	return k->grp[i] > k->grp[j];
}

/* Hoare partition with the first element as pivot, and the recursion of
 * src/bound_flowshop.cpp:597-625. The tie order of equal keys is whatever
 * this exact scheme produces, so it is restated step for step. */
static int hoare_partition(const fs_keys *k, int32_t *ord, int lo, int hi)
{
	int d = lo - 1, f = hi + 1;
	int32_t pivot = ord[lo];
	do {
		do {
			f--;
		} while (key_gt(k, ord[f], pivot));
		do {
			d++;
		} while (key_lt(k, ord[d], pivot));
		if (d < f) {
			int32_t t = ord[d];
			ord[d] = ord[f];
			ord[f] = t;
		}
	} while (d < f);
	return f;
}

static void hoare_sort(const fs_keys *k, int32_t *ord, int lo, int hi)
{
	if (hi - lo > 0) {
		int q = hoare_partition(k, ord, lo, hi);
		hoare_sort(k, ord, lo, q);
		hoare_sort(k, ord, q + 1, hi);
	}
}

fs_bound *fs_bound_create(const int32_t *p, int n, int m)
{
	if (n < 2 || n > FS_MAX_JOBS || m < 2 || m > FS_MAX_MACHINES)
		return NULL;
	fs_bound *b = (fs_bound *)calloc(1, sizeof(fs_bound));
	int P = m * (m - 1) / 2;
	b->n = n;
	b->m = m;
	b->P = P;
	b->p = (int32_t *)malloc(sizeof(int32_t) * m * n);
	memcpy(b->p, p, sizeof(int32_t) * m * n);
	b->mach[0] = (int32_t *)malloc(sizeof(int32_t) * P);
	b->mach[1] = (int32_t *)malloc(sizeof(int32_t) * P);
	b->lag = (int32_t *)malloc(sizeof(int32_t) * P * n);
	b->johnson = (int32_t *)malloc(sizeof(int32_t) * P * n);
	b->min_arr = (int32_t *)malloc(sizeof(int32_t) * m);
	b->min_dep = (int32_t *)malloc(sizeof(int32_t) * m);

	/* heads / tails: minimum over all jobs (remplirTempsArriverDepart) */
	b->min_arr[0] = 0;
	b->min_dep[m - 1] = 0;
	for (int k = 1; k < m; k++) {
		int32_t best = INT32_MAX;
		for (int j = 0; j < n; j++) {
			int32_t s = 0;
			for (int q = 0; q < k; q++)
				s += p[q * n + j];
			if (s < best)
				best = s;
		}
		b->min_arr[k] = best;
	}
	for (int k = 0; k < m - 1; k++) {
		int32_t best = INT32_MAX;
		for (int j = 0; j < n; j++) {
			int32_t s = 0;
			for (int q = k + 1; q < m; q++)
				s += p[q * n + j];
			if (s < best)
				best = s;
		}
		b->min_dep[k] = best;
	}

	/* pairs in lexicographic order (remplirMachine), lags (remplirLag) */
	int c = 0;
	for (int i = 0; i < m - 1; i++)
		for (int j = i + 1; j < m; j++) {
			b->mach[0][c] = i;
			b->mach[1][c] = j;
			c++;
		}
	for (int i = 0; i < P; i++) {
		int m1 = b->mach[0][i], m2 = b->mach[1][i];
		for (int j = 0; j < n; j++) {
			int32_t s = 0;
			for (int k = m1 + 1; k < m2; k++)
				s += p[k * n + j];
			b->lag[i * n + j] = s;
		}
	}

	/* Johnson orders (remplirTabJohnson / Johnson) */
	int32_t grp[FS_MAX_JOBS], key[FS_MAX_JOBS];
	fs_keys ks = {grp, key};
	for (int i = 0; i < P; i++) {
		int m1 = b->mach[0][i], m2 = b->mach[1][i];
		int32_t *ord = b->johnson + (int64_t)i * n;
		for (int j = 0; j < n; j++) {
			ord[j] = j;
			if (p[m1 * n + j] < p[m2 * n + j]) {
				grp[j] = 1;
				key[j] = p[m1 * n + j] + b->lag[i * n + j];
			} else {
				grp[j] = 2;
				key[j] = p[m2 * n + j] + b->lag[i * n + j];
			}
		}
		hoare_sort(&ks, ord, 0, n - 1);
	}
	return b;
}

void fs_bound_destroy(fs_bound *b)
{
	if (!b)
		return;
	free(b->p);
	free(b->mach[0]);
	free(b->mach[1]);
	free(b->lag);
	free(b->johnson);
	free(b->min_arr);
	free(b->min_dep);
	free(b);
}

int fs_bound_pairs(const fs_bound *b) { return b->P; }

void fs_bound_tables(const fs_bound *b, int32_t *mach0, int32_t *mach1,
                     int32_t *lag, int32_t *johnson, int32_t *min_arr,
                     int32_t *min_dep)
{
	int P = b->P, n = b->n, m = b->m;
	if (mach0)
		memcpy(mach0, b->mach[0], sizeof(int32_t) * P);
	if (mach1)
		memcpy(mach1, b->mach[1], sizeof(int32_t) * P);
	if (lag)
		memcpy(lag, b->lag, sizeof(int32_t) * P * n);
	if (johnson)
		memcpy(johnson, b->johnson, sizeof(int32_t) * P * n);
	if (min_arr)
		memcpy(min_arr, b->min_arr, sizeof(int32_t) * m);
	if (min_dep)
		memcpy(min_dep, b->min_dep, sizeof(int32_t) * m);
}

/* ------------------------------------------------------------------ */
/* Per-node bound (src/bound_flowshop.cpp:841-951)                     */
/* ------------------------------------------------------------------ */

static inline int32_t imax(int32_t a, int32_t b) { return a > b ? a : b; }

/* criteres_calculer (:897-909) */
int32_t fs_makespan(const fs_bound *b, const int32_t *perm)
{
	int n = b->n, m = b->m;
	int32_t t[FS_MAX_MACHINES];
	for (int k = 0; k < m; k++)
		t[k] = 0;
	for (int j = 0; j < n; j++) {
		int job = perm[j];
		t[0] += b->p[job];
		for (int k = 1; k < m; k++)
			t[k] = imax(t[k], t[k - 1]) + b->p[k * n + job];
	}
	return t[m - 1];
}

typedef struct {
	int32_t front[FS_MAX_MACHINES]; /* tempsMachines */
	int32_t back[FS_MAX_MACHINES];  /* tempsMachinesFin */
	uint8_t sched[FS_MAX_JOBS];     /* job[] != 0 */
	int f, nb;                      /* nbAffectDebut, nbAffectFin */
} fs_node;

/* set_tempsMachines_retardDebut (:841-856), set_job_jobFin (:858-868),
 * set_nombres (:870-874), set_tempsMachinesFin_tempsJobFin (:876-895). */
static void node_setup(const fs_bound *b, const int32_t *perm, int l1, int l2,
                       fs_node *s)
{
	int n = b->n, m = b->m;
	for (int k = 0; k < m; k++)
		s->front[k] = 0;
	for (int j = 0; j <= l1; j++) {
		int job = perm[j];
		s->front[0] += b->p[job];
		for (int k = 1; k < m; k++)
			s->front[k] = imax(s->front[k], s->front[k - 1]) + b->p[k * n + job];
	}
	memset(s->sched, 0, (size_t)n);
	for (int j = 0; j <= l1; j++)
		s->sched[perm[j]] = 1;
	for (int j = l2; j < n; j++)
		s->sched[perm[j]] = 1;
	s->f = l1 + 1;
	s->nb = n - l2;
	/* back times per start machine: makespan of perm[l2..n-1] on
	 * machines k..m-1, each recomputed from zero as the reference does */
	int32_t tmp[FS_MAX_MACHINES];
	for (int k0 = m - 1; k0 >= 0; k0--) {
		for (int k = k0; k < m; k++)
			tmp[k] = 0;
		for (int j = l2; j < n; j++) {
			int job = perm[j];
			tmp[k0] += b->p[k0 * n + job];
			for (int k = k0 + 1; k < m; k++)
				tmp[k] = imax(tmp[k - 1], tmp[k]) + b->p[k * n + job];
		}
		s->back[k0] = tmp[m - 1];
	}
}

/* initCmax + heuristiqueCmax + cmaxFin for one pair (:64-100, :136-149) */
static int32_t pair_value(const fs_bound *b, const fs_node *s, int i)
{
	int n = b->n;
	int m1 = b->mach[0][i], m2 = b->mach[1][i];
	int32_t t0, t1;
	if (s->f != 0) {
		t0 = s->front[m1];
		t1 = s->front[m2];
	} else {
		t0 = b->min_arr[m1];
		t1 = b->min_arr[m2];
	}
	const int32_t *ord = b->johnson + (int64_t)i * n;
	const int32_t *lag = b->lag + (int64_t)i * n;
	const int32_t *p1 = b->p + (int64_t)m1 * n;
	const int32_t *p2 = b->p + (int64_t)m2 * n;
	for (int q = 0; q < n; q++) {
		int j = ord[q];
		if (!s->sched[j]) {
			t0 += p1[j];
			t1 = imax(t1, t0 + lag[j]) + p2[j];
		}
	}
	if (s->nb != 0)
		t1 = imax(t1 + s->back[m2], t0 + s->back[m1]);
	else
		t1 += b->min_dep[m2];
	return t1;
}

/* bornes_calculer (:929-946) -> calculBorne -> borneInfMakespan (:121-168).
 * moinsBon starts at 0, is raised on a strict '>' (first binding pair wins
 * ties), and the early exit fires when moinsBon > best, best != -1. */
int32_t fs_bound_eval(const fs_bound *b, const int32_t *perm, int l1, int l2,
                      int32_t best, int32_t *argmax)
{
	if (l2 - l1 == 1) {
		if (argmax)
			*argmax = -1;
		return fs_makespan(b, perm);
	}
	fs_node s;
	node_setup(b, perm, l1, l2, &s);
	int32_t lb = 0, arg = -1;
	for (int i = 0; i < b->P; i++) {
		int32_t v = pair_value(b, &s, i);
		if (v > lb) {
			lb = v;
			arg = i;
		}
		if (lb > best && best != -1)
			break;
	}
	if (argmax)
		*argmax = arg;
	return lb;
}

int32_t fs_bound_eval_pairs(const fs_bound *b, const int32_t *perm, int l1,
                            int l2, const int32_t *pairs, int npairs)
{
	if (l2 - l1 == 1)
		return fs_makespan(b, perm);
	fs_node s;
	node_setup(b, perm, l1, l2, &s);
	int32_t lb = 0;
	for (int q = 0; q < npairs; q++) {
		int32_t v = pair_value(b, &s, pairs[q]);
		if (v > lb)
			lb = v;
	}
	return lb;
}

/* LB1: for every machine k, head_k + remaining work on k + tail_k, with
 * the reference's head/tail conventions (front time if jobs are fixed at
 * the front, else the static head; back time if jobs are fixed at the
 * back, else the static tail). Not present in the reference. */
int32_t fs_lb1_eval(const fs_bound *b, const int32_t *perm, int l1, int l2)
{
	if (l2 - l1 == 1)
		return fs_makespan(b, perm);
	int n = b->n, m = b->m;
	fs_node s;
	node_setup(b, perm, l1, l2, &s);
	int32_t lb = 0;
	for (int k = 0; k < m; k++) {
		int32_t h = s.f ? s.front[k] : b->min_arr[k];
		int32_t t = s.nb ? s.back[k] : b->min_dep[k];
		int32_t w = 0;
		for (int j = 0; j < n; j++)
			if (!s.sched[j])
				w += b->p[k * n + j];
		int32_t v = h + w + t;
		if (v > lb)
			lb = v;
	}
	return lb;
}

typedef struct {
	const fs_bound *b;
	const int32_t *perms, *l1, *l2;
	int32_t *out, *arg;
	int64_t lo, hi;
} batch_job;

static void *batch_worker(void *arg)
{
	batch_job *j = (batch_job *)arg;
	int n = j->b->n;
	for (int64_t r = j->lo; r < j->hi; r++) {
		int32_t a;
		j->out[r] = fs_bound_eval(j->b, j->perms + r * n, j->l1[r], j->l2[r],
		                          -1, &a);
		if (j->arg)
			j->arg[r] = a;
	}
	return NULL;
}

void fs_bound_eval_batch(const fs_bound *b, const int32_t *perms,
                         const int32_t *l1, const int32_t *l2, int64_t count,
                         int32_t *out, int32_t *arg, int nthreads)
{
	if (nthreads <= 1 || count < 2 * nthreads) {
		batch_job j = {b, perms, l1, l2, out, arg, 0, count};
		batch_worker(&j);
		return;
	}
	if (nthreads > 256)
		nthreads = 256;
	pthread_t th[256];
	batch_job jobs[256];
	for (int t = 0; t < nthreads; t++) {
		jobs[t] = (batch_job){b, perms, l1, l2, out, arg,
		                      count * t / nthreads, count * (t + 1) / nthreads};
		pthread_create(&th[t], NULL, batch_worker, &jobs[t]);
	}
	for (int t = 0; t < nthreads; t++)
		pthread_join(th[t], NULL);
}

void fs_lb1_eval_batch(const fs_bound *b, const int32_t *perms,
                       const int32_t *l1, const int32_t *l2, int64_t count,
                       int32_t *out)
{
	for (int64_t r = 0; r < count; r++)
		out[r] = fs_lb1_eval(b, perms + r * b->n, l1[r], l2[r]);
}

/* ------------------------------------------------------------------ */
/* NEH (initial upper bound; not in the reference)                     */
/* ------------------------------------------------------------------ */

static int32_t seq_makespan(const int32_t *p, int n, int m, const int32_t *seq,
                            int len)
{
	int32_t t[FS_MAX_MACHINES];
	for (int k = 0; k < m; k++)
		t[k] = 0;
	for (int q = 0; q < len; q++) {
		int job = seq[q];
		t[0] += p[job];
		for (int k = 1; k < m; k++)
			t[k] = imax(t[k], t[k - 1]) + p[k * n + job];
	}
	return t[m - 1];
}

/* Jobs by decreasing total work (ties: lower index first); each job is
 * inserted at the first position giving the smallest partial makespan. */
int32_t fs_neh(const int32_t *p, int n, int m, int32_t *perm_out)
{
	int32_t order[FS_MAX_JOBS], tot[FS_MAX_JOBS];
	for (int j = 0; j < n; j++) {
		order[j] = j;
		tot[j] = 0;
		for (int k = 0; k < m; k++)
			tot[j] += p[k * n + j];
	}
	for (int a = 1; a < n; a++) { /* stable insertion sort */
		int32_t x = order[a];
		int c = a - 1;
		while (c >= 0 && tot[order[c]] < tot[x]) {
			order[c + 1] = order[c];
			c--;
		}
		order[c + 1] = x;
	}
	int32_t seq[FS_MAX_JOBS], cand[FS_MAX_JOBS];
	int len = 0;
	for (int a = 0; a < n; a++) {
		int32_t job = order[a];
		int32_t best = INT32_MAX;
		int bpos = 0;
		for (int pos = 0; pos <= len; pos++) {
			int w = 0;
			for (int q = 0; q < pos; q++)
				cand[w++] = seq[q];
			cand[w++] = job;
			for (int q = pos; q < len; q++)
				cand[w++] = seq[q];
			int32_t c = seq_makespan(p, n, m, cand, len + 1);
			if (c < best) {
				best = c;
				bpos = pos;
			}
		}
		for (int q = len; q > bpos; q--)
			seq[q] = seq[q - 1];
		seq[bpos] = job;
		len++;
	}
	memcpy(perm_out, seq, sizeof(int32_t) * n);
	return seq_makespan(p, n, m, seq, n);
}

/* ------------------------------------------------------------------ */
/* DFS explorer (src/explorer.cu:92-148 with decompose_beginend)       */
/* ------------------------------------------------------------------ */

typedef struct {
	int32_t perm[FS_MAX_JOBS];
	int16_t l1, l2, depth, pad;
	int32_t lb;  /* couts[0] == couts_somme */
	int32_t job; /* job moved by the last branching (rank tie-break) */
} ex_node;

typedef struct {
	ex_node *v;
	int64_t size, cap;
} ex_stack;

static int st_push(ex_stack *s, const ex_node *x)
{
	if (s->size == s->cap) {
		int64_t nc = s->cap ? s->cap * 2 : 1024;
		ex_node *nv = (ex_node *)realloc(s->v, sizeof(ex_node) * nc);
		if (!nv)
			return -1;
		s->v = nv;
		s->cap = nc;
	}
	s->v[s->size++] = *x;
	return 0;
}

/* create_raw_problem3 (src/bb_problem_calculator.cpp:25-79) */
static void make_child(const ex_node *fa, int indice, int begin_end, int n,
                       int father_simple, ex_node *c)
{
	c->l1 = fa->l1;
	c->l2 = fa->l2;
	if (begin_end == 0)
		c->l1++;
	else
		c->l2--;
	if (c->l2 - c->l1 == 2)
		c->l1++;
	c->depth = father_simple ? (int16_t)n : (int16_t)(fa->depth + 1);
	c->job = fa->perm[indice];
	memcpy(c->perm, fa->perm, sizeof(int32_t) * n);
	int slot = begin_end == 0 ? fa->l1 + 1 : fa->l2 - 1;
	int32_t t = c->perm[slot];
	c->perm[slot] = c->perm[indice];
	c->perm[indice] = t;
}

/* select_worst (src/select_worst.cpp:7-12): descending LB, ties by
 * descending job; rank 0 goes to the last element (problems::ranks). */
static int worse_first(const ex_node *a, const ex_node *b)
{
	if (a->lb != b->lb)
		return b->lb < a->lb;
	return a->job > b->job;
}

static void sort_worst_first(ex_node *v, int cnt)
{
	for (int a = 1; a < cnt; a++) {
		ex_node x = v[a];
		int c = a - 1;
		while (c >= 0 && worse_first(&x, &v[c])) {
			v[c + 1] = v[c];
			c--;
		}
		v[c + 1] = x;
	}
}

static void add_coverage(fs_stats *st, int n, int depth)
{
	/* weights::depths[d] = (n-d)! (weights.cpp), summed by the caller */
	(void)n;
	st->depth_hist[depth]++;
}

/* The take loop of explorer::_explore_cpu over a stack that already holds
 * the starting nodes (the root, or seeded open nodes); frees the stack. */
static int explore_core(const fs_bound *b, ex_stack S, int32_t ub0, int32_t best,
                        int64_t node_cap, fs_stats *st, int32_t *best_perm,
                        fs_log_cb log_cb, fs_pair_sel_cb pair_sel, void *user)
{
	int n = b->n;
	memset(st, 0, sizeof(*st));
	int32_t ub = ub0; /* the incumbent list's minimum; INT32_MAX = empty */
	ex_node *kids = (ex_node *)malloc(sizeof(ex_node) * 2 * n);
	int32_t sel[FS_MAX_MACHINES * FS_MAX_MACHINES];
	int64_t takes = 0;
	int rc = 0;
	while (S.size > 0) {
		if (node_cap && takes >= node_cap) {
			rc = 1;
			break;
		}
		ex_node nd = S.v[--S.size];
		takes++;
		if (nd.depth == n) {
			/* leaf: solutions::insert; inserable iff cost < every
			 * incumbent (eliminate_pareto) */
			st->leaves++;
			if (nd.lb < ub) {
				ub = nd.lb;
				st->improved++;
				if (best_perm)
					memcpy(best_perm, nd.perm, sizeof(int32_t) * n);
			}
			add_coverage(st, n, nd.depth);
			continue;
		}
		if (!(nd.lb < ub)) { /* solutions::inserable fails -> pruned */
			st->pruned++;
			add_coverage(st, n, nd.depth);
			continue;
		}
		st->branched++;
		int simple = nd.depth == n - 2;
		int cnt = 0;
		if (simple) {
			/* leaves_generate (decompose_beginend.cpp:70-89) */
			for (int q = 1; q <= 2; q++) {
				ex_node *c = &kids[cnt++];
				make_child(&nd, nd.l1 + q, 0, n, 1, c);
				c->lb = fs_makespan(b, c->perm);
			}
			st->bounded += 2;
			sort_worst_first(kids, cnt);
		} else {
			/* problems_generate for BEGIN then END (:26-68) */
			int u = nd.l2 - nd.l1 - 1;
			int64_t sum[2] = {0, 0}, cut[2] = {0, 0};
			for (int side = 0; side < 2; side++)
				for (int j = nd.l1 + 1; j < nd.l2; j++) {
					ex_node *c = &kids[cnt++];
					make_child(&nd, j, side, n, 0, c);
					int32_t arg = -1;
					int settled = 0;
					if (pair_sel) {
						int np = pair_sel(c->perm, c->l1, c->l2, sel, user);
						if (np > 0) {
							int32_t part = fs_bound_eval_pairs(b, c->perm, c->l1,
							                                   c->l2, sel, np);
							if (part >= best) {
								c->lb = part;
								settled = 1;
								st->early_exits++;
							}
						}
					}
					if (!settled)
						c->lb = fs_bound_eval(b, c->perm, c->l1, c->l2, 999999,
						                      &arg);
					if (log_cb && !settled)
						log_cb(c->perm, c->l1, c->l2, arg, c->lb, user);
					if (c->lb >= best)
						cut[side]++;
					else
						sum[side] += c->lb;
				}
			st->bounded += 2 * u;
			/* choise (:39-50): more cut children wins, else larger sum
			 * wins, ties go to END */
			int side;
			if (cut[0] > cut[1])
				side = 0;
			else if (cut[1] > cut[0])
				side = 1;
			else
				side = (sum[0] > sum[1]) ? 0 : 1;
			ex_node *chosen = kids + side * u;
			if (side == 1)
				memmove(kids, chosen, sizeof(ex_node) * u);
			cnt = u;
			sort_worst_first(kids, cnt);
		}
		/* ranks: rank 0 = last element; the DFS pops the smallest rank
		 * path first (comparator_depth), so push worst first. */
		for (int q = 0; q < cnt; q++)
			if (st_push(&S, &kids[q])) {
				rc = -2;
				goto done;
			}
	}
done:
	st->best_cost = ub;
	free(kids);
	free(S.v);
	return rc;
}

int fs_explore(const fs_bound *b, int32_t ub0, int32_t best, int64_t node_cap,
               fs_stats *st, int32_t *best_perm, fs_log_cb log_cb,
               fs_pair_sel_cb pair_sel, void *user)
{
	int n = b->n;
	ex_stack S = {0, 0, 0};
	ex_node root;
	memset(&root, 0, sizeof(root));
	for (int j = 0; j < n; j++)
		root.perm[j] = j;
	root.l1 = -1;
	root.l2 = (int16_t)n;
	root.depth = 0;
	root.lb = 0;
	root.job = -1;
	if (st_push(&S, &root))
		return -2;
	return explore_core(b, S, ub0, best, node_cap, st, best_perm, log_cb, pair_sel, user);
}

int fs_explore_seeded(const fs_bound *b, const int32_t *perms, const int32_t *l1,
                      const int32_t *l2, const int32_t *lbs, int64_t count, int32_t ub0,
                      int32_t best, int64_t node_cap, fs_stats *st, int32_t *best_perm)
{
	int n = b->n;
	ex_stack S = {0, 0, 0};
	for (int64_t i = 0; i < count; i++) {
		ex_node x;
		memset(&x, 0, sizeof(x));
		memcpy(x.perm, perms + i * n, sizeof(int32_t) * n);
		x.l1 = (int16_t)l1[i];
		x.l2 = (int16_t)l2[i];
		x.depth = (int16_t)(n - (l2[i] - l1[i] - 1));
		x.lb = lbs[i];
		x.job = -1;
		if (st_push(&S, &x)) {
			free(S.v);
			return -2;
		}
	}
	return explore_core(b, S, ub0, best, node_cap, st, best_perm, NULL, NULL, NULL);
}

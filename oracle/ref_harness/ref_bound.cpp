// TEST INFRASTRUCTURE (oracle pin only): a C-ABI around the reference's own
// bound_flowshop (src/bound_flowshop.cpp, compiled unmodified from the
// reference tree). Used to generate golden vectors and to time the
// reference CPU bound in this container.
//
//   ref_bound_create(p, n, m)     bound_abstract::set_pbab + set_instance
//                                 (src/bound_abstract.cpp, bound_flowshop.cpp:953-956)
//   ref_bound_eval(...)           bornes_calculer(perm, l1, l2, couts, 999999)
//                                 (bound_flowshop.cpp:929-951); the binding
//                                 pair is read back from the reference's own
//                                 nbFois statistic (:157,:164)
#include <pthread.h>
#include <string.h>

#include "ref_common.hpp"

struct ref_bound_handle {
	pbab *pb;
	instance_abstract *inst;
	bound_flowshop *bound;
	int n, m, P;
};

// pbab has no default constructor and src/pbab.cpp is not linked; the bound
// only dereferences pbb->instance (bound_flowshop.cpp:320-335), so a zeroed
// object with that one field set is enough.
static pbab *ref_bare_pbab(instance_abstract *inst)
{
	pbab *pb = (pbab *)calloc(1, sizeof(pbab));
	pb->instance = inst;
	pb->size = inst->size;
	return pb;
}

extern "C" void *ref_bound_create(const int32_t *p, int n, int m)
{
	ref_bound_handle *h = new ref_bound_handle;
	h->inst = ref_make_instance(p, n, m);
	h->pb = ref_bare_pbab(h->inst);
	h->bound = new bound_flowshop();
	h->bound->set_pbab(h->pb);
	h->bound->set_instance(h->inst);
	h->n = n;
	h->m = m;
	h->P = m * (m - 1) / 2;
	return h;
}

extern "C" void ref_bound_destroy(void *hv)
{
	ref_bound_handle *h = (ref_bound_handle *)hv;
	// The reference never frees its bound tables; the handle is leaked on
	// purpose rather than guessing at its ownership rules.
	delete h;
}

static void eval_range(ref_bound_handle *h, const int32_t *perms,
                       const int32_t *l1, const int32_t *l2, int64_t lo,
                       int64_t hi, int32_t *out, int32_t *argmax)
{
	int n = h->n, P = h->P;
	int *perm = new int[n];
	int *before = new int[P];
	int couts[2];
	for (int64_t r = lo; r < hi; r++) {
		for (int j = 0; j < n; j++)
			perm[j] = perms[r * n + j];
		memcpy(before, h->bound->nbFois, sizeof(int) * P);
		h->bound->bornes_calculer(perm, l1[r], l2[r], couts, 999999);
		out[r] = couts[0];
		if (argmax) {
			int32_t a = -1;
			for (int i = 0; i < P; i++)
				if (h->bound->nbFois[i] != before[i]) {
					a = i;
					break;
				}
			argmax[r] = a;
		}
	}
	delete[] perm;
	delete[] before;
}

extern "C" void ref_bound_eval(void *hv, const int32_t *perms,
                               const int32_t *l1, const int32_t *l2,
                               int64_t count, int32_t *out, int32_t *argmax)
{
	eval_range((ref_bound_handle *)hv, perms, l1, l2, 0, count, out, argmax);
}

struct mt_job {
	ref_bound_handle *h;
	const int32_t *perms, *l1, *l2;
	int32_t *out;
	int64_t lo, hi;
};

static void *mt_worker(void *a)
{
	mt_job *j = (mt_job *)a;
	eval_range(j->h, j->perms, j->l1, j->l2, j->lo, j->hi, j->out, NULL);
	return NULL;
}

// Multi-threaded timing helper: bound_flowshop keeps per-object scratch
// (bound_flowshop.h:34-75) and is not re-entrant, so each thread gets its
// own object built from the same instance.
extern "C" void ref_bound_eval_mt(const int32_t *p, int n, int m,
                                  const int32_t *perms, const int32_t *l1,
                                  const int32_t *l2, int64_t count,
                                  int32_t *out, int nthreads)
{
	if (nthreads < 1)
		nthreads = 1;
	if (nthreads > 256)
		nthreads = 256;
	ref_bound_handle *hs[256];
	for (int t = 0; t < nthreads; t++)
		hs[t] = (ref_bound_handle *)ref_bound_create(p, n, m);
	pthread_t th[256];
	mt_job jobs[256];
	for (int t = 0; t < nthreads; t++) {
		jobs[t].h = hs[t];
		jobs[t].perms = perms;
		jobs[t].l1 = l1;
		jobs[t].l2 = l2;
		jobs[t].out = out;
		jobs[t].lo = count * t / nthreads;
		jobs[t].hi = count * (t + 1) / nthreads;
		pthread_create(&th[t], NULL, mt_worker, &jobs[t]);
	}
	for (int t = 0; t < nthreads; t++)
		pthread_join(th[t], NULL);
}

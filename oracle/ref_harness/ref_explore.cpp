// TEST INFRASTRUCTURE (oracle pin only): runs the reference's CPU search on
// one instance through the reference's own objects — tree (priority queue
// by rank path, src/tree.cpp), decompose_beginend (src/decompose_beginend.cpp),
// problems / select_worst ranks, bb_problem_calculator children,
// bound_flowshop, solutions + eliminate_pareto incumbent, weights coverage —
// and prints the reference's counters.
//
// The take loop restates explorer::_explore_cpu (src/explorer.cu:92-148)
// without its socket hooks (sendOptimalSolutionToGPUs, pendingWorkRequest)
// and without the 250-take slicing, which only interleaves protocol work.
// The initial upper bound goes in through the reference's own path: a
// bab.solutions record in the working directory read by solutions::init
// (src/solutions.cpp:26-35, 69-86).
//
// usage: ref_explore <n> <m> <ub0|-1> <best> <workdir/> [taillard_id]
//   processing times (m*n ints, machine-major) on stdin unless a Taillard
//   id is given, in which case the reference generator
//   (src/instance_flowshop.cpp:74-96) makes the instance.
// Last line of output: RESULT {json}
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <fstream>
#include <iostream>
#include <vector>

#include "ref_common.hpp"
#include "decompose_beginend.h"
#include "eliminate_abstract.h"
#include "eliminate_pareto.h"
#include "instance_abstract.h"
#include "instance_flowshop.h"
#include "problems.h"
#include "solutions.h"
#include "tree.h"
#include "weights.h"

// Static members the reference defines in src/arguments.cpp:6-35.
char arguments::directory[50];
char arguments::worker_name[50];
char arguments::file[50];
int arguments::worker_port;
char arguments::type = 'c';
char arguments::gpu_mode;
char arguments::index_name[50];
int arguments::index_port;
bool arguments::worker = true;
bool arguments::root = false;
int arguments::sizev;
int arguments::instancev;
int arguments::costv;
int arguments::checkpointv;
int arguments::balancingv;
bool arguments::divisionv;
int arguments::cpu_number = 0;
int arguments::gpu_number = 0;
int arguments::explorer_number = 0;
int arguments::pool_number = 0;
int arguments::pool_size = 0;
int arguments::sleep_number = 0;
int arguments::period = 0;
bool arguments::file_exists = false;
char arguments::johnson = 'g';
char arguments::temps = 'p';
char arguments::divergence = 'v';
char arguments::strategy = STRATEGY_DEPTH;
int arguments::devices = -1;
int arguments::cpu_operation = CPU_NOT_DEFINED;

// The part of pbab::pbab (src/pbab.cpp:30-80) that the CPU search uses:
// weights, decomposition, bound, tree and incumbent lists. Peers, the GPU
// pool, works and the explorer object are socket / GPU runtime and are not
// built here.
pbab::pbab(int, int, int, eliminate_abstract *_eliminate,
           decompose_beginend *_decompose, instance_abstract *_instance,
           bound_abstract *_bound, tree *_tr)
{
	size = arguments::sizev;
	wghts = new weights(this);
	pr = ndx = NULL;
	eliminate = _eliminate;
	decompose = _decompose;
	instance = _instance;
	bound = _bound;
	select = NULL;
	ttm = NULL;
	decompose->set_pbab(this);
	decompose->set_bound(bound);
	bound->set_pbab(this);
	bound->set_instance(instance);
	xplr = NULL;
	if (_tr)
		_tr->set_pbab(this);
	tr = _tr;
	isltns = new solutions(arguments::directory, this);
	wsltns = new solutions(arguments::directory, this);
	wrks = NULL;
	sltn = NULL;
	gp = NULL;
	cpu_operation = arguments::cpu_operation;
	node = NULL;
}

int main(int argc, char **argv)
{
	if (argc < 6) {
		fprintf(stderr, "usage: ref_explore n m ub0 best workdir/ [taillard_id]\n");
		return 2;
	}
	int n = atoi(argv[1]), m = atoi(argv[2]);
	int ub0 = atoi(argv[3]);
	int best = atoi(argv[4]);
	strncpy(arguments::directory, argv[5], 49);
	arguments::sizev = n;
	arguments::costv = 9999999; // arguments::initialization, non-optimal mode

	instance_abstract *inst;
	if (argc > 6) {
		inst = new instance_flowshop(atoi(argv[6]));
	} else {
		std::vector<int32_t> p((size_t)n * m);
		for (size_t i = 0; i < p.size(); i++)
			if (scanf("%d", &p[i]) != 1) {
				fprintf(stderr, "short instance on stdin\n");
				return 2;
			}
		inst = ref_make_instance(p.data(), n, m);
	}

	if (ub0 >= 0) {
		// one incumbent record: couts[2] couts_somme perm[MAX_NBJOBS]
		// limite1 limite2 depth job begin_end (bb_problem_calculator.cpp:101-126)
		std::ofstream f((std::string(arguments::directory) + "bab.solutions").c_str());
		f << 1 << " " << ub0 << " 0 " << ub0 << " ";
		for (int j = 0; j < WSBB_SHIM_MAXJOBS; j++)
			f << (j < n ? j : 0) << " ";
		f << (n - 1) << " " << n << " " << n << " " << -1 << " " << 0 << "\n";
	}

	tree *tr = new tree(STRATEGY_DEPTH);
	decompose_beginend *dec = new decompose_beginend(best);
	bound_flowshop *bnd = new bound_flowshop();
	eliminate_pareto *elim = new eliminate_pareto();
	pbab *pbb = new pbab(1, 1, 0, elim, dec, inst, bnd, tr);
	dec->ns.bbCalculator = tr->bbCalculator;

	tr->add_root(); // tree.cpp:170-176
	pbb->wsltns->init(); // reads bab.solutions, sets the incumbent
	long improved_at_start = 0;
	for (solutions::iterator i = pbb->wsltns->begin(); i != pbb->wsltns->end(); ++i)
		improved_at_start++;

	long branched = 0, pruned = 0, leaves = 0, bounded = 0, improved = 0;
	BigInteger coverage(0);
	while (true) {
		raw_bb_problem *nd = tr->take();
		if (!nd)
			break;
		if (tr->bbCalculator->leaf(nd)) {
			if (pbb->wsltns->insert(nd))
				improved++;
			leaves++;
			coverage += pbb->wghts->depths[nd->depth];
		} else if (pbb->wsltns->inserable(nd)) {
			bounded += tr->bbCalculator->simple(nd) ? 2 : 2 * (nd->limite2 - nd->limite1 - 1);
			tr->insert((*pbb->decompose)(*nd));
			branched++;
		} else {
			pruned++;
			coverage += pbb->wghts->depths[nd->depth];
		}
		free(nd);
	}
	int bestc = -1;
	std::vector<int> bestperm;
	for (solutions::iterator i = pbb->wsltns->begin(); i != pbb->wsltns->end(); ++i) {
		bestc = i->couts_somme;
		bestperm.assign(i->permutation, i->permutation + n);
	}
	std::cout << "RESULT {\"n\": " << n << ", \"m\": " << m << ", \"ub0\": " << ub0
	          << ", \"best\": " << best << ", \"branched\": " << branched
	          << ", \"pruned\": " << pruned << ", \"leaves\": " << leaves
	          << ", \"improved\": " << improved << ", \"preloaded\": " << improved_at_start
	          << ", \"bounded\": " << bounded << ", \"optimum\": " << bestc
	          << ", \"coverage\": \"" << easyBItoString(coverage) << "\", \"perm\": [";
	for (size_t j = 0; j < bestperm.size(); j++)
		std::cout << (j ? ", " : "") << bestperm[j];
	std::cout << "]}" << std::endl;
	return 0;
}

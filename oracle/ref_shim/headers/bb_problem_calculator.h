// Test infrastructure (oracle pin only): stand-in for the reference's
// headers/bb_problem_calculator.h, which the reference includes but does
// not ship. The layout of raw_bb_problem is inferred from its uses:
//   src/bb_problem_calculator.cpp:9-33 (fields set on create),
//   src/bb_problem_calculator.cpp:101-144 (stream order: couts[2],
//   couts_somme, permutation[MAX_NBJOBS], limite1, limite2, depth, job,
//   begin_end), src/gpu.cu:269-271 (couts / couts_somme writes),
//   src/tree.cpp:37-46 (ranks[MAX_NBJOBS + 1]).
// cpu_raw_bb_problem follows src/work_stealing/protocol.cpp:208-211.
// The class declaration mirrors the member definitions in
// src/bb_problem_calculator.cpp.
#ifndef BB_PROBLEM_CALCULATOR_H
#define BB_PROBLEM_CALCULATOR_H

#include <iostream>

#ifndef WSBB_SHIM_MAXJOBS
#define WSBB_SHIM_MAXJOBS 20
#endif

#ifndef BEGIN_ORDER
#define BEGIN_ORDER 0
#endif
#ifndef END_ORDER
#define END_ORDER 1
#endif

struct raw_bb_problem {
	int couts[2];
	int couts_somme;
	int permutation[WSBB_SHIM_MAXJOBS];
	int ranks[WSBB_SHIM_MAXJOBS + 1];
	int limite1;
	int limite2;
	int depth;
	int job;
	int begin_end;
};

struct cpu_raw_bb_problem {
	raw_bb_problem *data;
	int size_int_byte;
};

class pbab;

class bb_problem_calculator {
public:
	pbab *pbb;
	bb_problem_calculator(pbab *pbb);
	raw_bb_problem *create_raw_problem(pbab *pbb);
	void create_raw_problem3(const raw_bb_problem *father, int indice,
	                         int begin_end, raw_bb_problem *child);
	void free_raw_problem(raw_bb_problem *p);
	void limites_set(const raw_bb_problem *father, raw_bb_problem *child,
	                 int begin_end);
	bool simple(const raw_bb_problem *p);
	bool leaf(const raw_bb_problem *p);
	void depth_set(const raw_bb_problem *father, raw_bb_problem *child);
	void permutation_set(const raw_bb_problem *father, int indice,
	                     int begin_end, raw_bb_problem *child);
	void ranks_set(const raw_bb_problem *father, raw_bb_problem *child);
	void ranks_depth(raw_bb_problem *child, int rank);
	void ranks_depth2(raw_bb_problem *child, int rank);
	void print(raw_bb_problem *p);
};

std::istream &operator>>(std::istream &stream, raw_bb_problem &p);
std::ostream &operator<<(std::ostream &stream, raw_bb_problem &p);

#endif

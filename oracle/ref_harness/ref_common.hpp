// TEST INFRASTRUCTURE (oracle pin only). Shared set-up for the harnesses
// that drive the reference's own compiled translation units (built in place
// from the reference's src/ by oracle/build.sh; nothing from the
// reference is copied into this repository).
//
// What the reference's src/pbab.cpp:30-80 and src/arguments.cpp:6-35 would
// provide is defined here instead, restricted to what the bound, the
// decomposition, the tree and the incumbent list touch; pbab.cpp itself
// pulls in the socket runtime and is not linked.
#ifndef WSBB_REF_COMMON_HPP
#define WSBB_REF_COMMON_HPP

#include <stdint.h>
#include <sstream>
#include <string>

#include "bound_flowshop.h"
#include "instance_abstract.h"
#include "pbab.h"

// Text stream in the reference instance format "n m seed p[m][n]"
// (src/instance_flowshop.cpp:84-89), machine-major.
inline std::stringstream *ref_instance_stream(const int32_t *p, int n, int m)
{
	std::stringstream *s = new std::stringstream();
	*s << n << " " << m << " " << 0 << " ";
	for (int k = 0; k < m; k++)
		for (int j = 0; j < n; j++)
			*s << p[k * n + j] << " ";
	return s;
}

inline instance_abstract *ref_make_instance(const int32_t *p, int n, int m)
{
	instance_abstract *inst = new instance_abstract;
	inst->size = n;
	inst->data = ref_instance_stream(p, n, m);
	return inst;
}

#endif

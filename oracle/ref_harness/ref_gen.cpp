// TEST INFRASTRUCTURE (oracle pin only). The reference's own time draw,
// instance_flowshop::unif (src/instance_flowshop.cpp:74-82), called in the
// order of its generate_instance (:84-89: machine-major, times in [1, 99])
// for a caller-given time seed instead of a benchmark id.
#include <stdint.h>
#include <new>

#include "instance_abstract.h"
#include "instance_flowshop.h"

extern "C" void ref_taillard(long seed, int n, int m, int32_t *p)
{
	// unif reads no member: storage of the right size stands in for an
	// object (the constructor would generate a benchmark instance)
	void *raw = ::operator new(sizeof(instance_flowshop));
	instance_flowshop *gen = static_cast<instance_flowshop *>(raw);
	long s = seed;
	for (int k = 0; k < m; k++)
		for (int j = 0; j < n; j++)
			p[k * n + j] = (int32_t)gen->unif(&s, 1, 99);
	::operator delete(raw);
}

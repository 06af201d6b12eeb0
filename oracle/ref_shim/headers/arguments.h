// Test infrastructure (oracle pin only): stand-in for the reference's
// headers/arguments.h, which the reference includes but does not ship.
// It declares the static-member class whose definitions live in the
// reference's src/arguments.cpp:6-35 (same member names and types).
// The harnesses under oracle/ref_harness define these statics themselves,
// so src/arguments.cpp (which reads ../parameters files) is never linked.
#ifndef ARGUMENTS_H
#define ARGUMENTS_H

#include <getopt.h>
#include <string.h>

class arguments {
public:
	static char directory[50];
	static char worker_name[50];
	static char file[50];
	static int worker_port;
	static char type;
	static char gpu_mode;
	static char index_name[50];
	static int index_port;
	static bool worker;
	static bool root;
	static int sizev;
	static int instancev;
	static int costv;
	static int checkpointv;
	static int balancingv;
	static bool divisionv;
	static int cpu_number;
	static int gpu_number;
	static int explorer_number;
	static int pool_number;
	static int pool_size;
	static int sleep_number;
	static int period;
	static bool file_exists;
	static char johnson;
	static char temps;
	static char divergence;
	static char strategy;
	static int devices;
	static int cpu_operation;

	static void initialization(int instance, bool optimal);
	static void parse_arguments(int argc, char **argv);
};

#endif

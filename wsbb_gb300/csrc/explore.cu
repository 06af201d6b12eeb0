// Exact begin-end DFS search on the GPU (filled in below the pool path).
#include "wsbb_internal.h"

void wsbb_explore_release(wsbb_ctx *ctx) { (void)ctx; }

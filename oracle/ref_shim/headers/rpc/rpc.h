// Test infrastructure (oracle pin only): empty stand-in for the reference's
// missing rpc/rpc.h (included from headers/peer.h:8); nothing on the bound
// or explorer path uses it.

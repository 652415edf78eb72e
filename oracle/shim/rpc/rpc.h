/* Stand-in for SunRPC <rpc/rpc.h>.  Test infrastructure only. */
#include "types.h"
#include "xdr.h"

/* Stand-in for SunRPC <rpc/types.h>, for the reference's snapshot I/O.
 * Test infrastructure only. */
#ifndef TSPH_SHIM_RPC_TYPES_H
#define TSPH_SHIM_RPC_TYPES_H
typedef int bool_t;
typedef unsigned int u_int;
typedef int enum_t;
typedef char *caddr_t;
#ifndef TRUE
#define TRUE 1
#endif
#ifndef FALSE
#define FALSE 0
#endif
#endif

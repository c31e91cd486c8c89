/* Minimal stand-in for the CANN runtime header, just enough for the
 * reference's API layer (lib/*.cpp) to compile on a machine without CANN.
 * Used only by oracle/Makefile to build the reference's plan/validation
 * layer as an error-code oracle. */
#ifndef ORACLE_STUB_ACL_H
#define ORACLE_STUB_ACL_H
typedef void* aclrtStream;
typedef int aclError;
#define ACL_SUCCESS 0
#define ACL_ERROR_INVALID_PARAM 100000
#endif

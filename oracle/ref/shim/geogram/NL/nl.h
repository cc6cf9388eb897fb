/* Build shim for the oracle's reference library.  The reference's NL/nl.h
 * forwards to the OpenNL submodule, which is empty in the checkout.  The
 * kd-tree and convex-cell code never call OpenNL; only
 * basic/command_line.cpp:697-698 names these two entry points, so this
 * header declares them and nl_stub.c defines them as no-ops. */
#ifndef GBV_REF_NL_SHIM_H
#define GBV_REF_NL_SHIM_H
#ifdef __cplusplus
extern "C" {
#endif
typedef int (*NLprintfFunc)(const char* format, ...);
typedef int (*NLfprintfFunc)(FILE* out, const char* format, ...);
void nlPrintfFuncs(NLprintfFunc f1, NLfprintfFunc f2);
void nlInitialize(int argc, char** argv);
#ifdef __cplusplus
}
#endif
#endif

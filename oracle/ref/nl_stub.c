/* No-op definitions for the two OpenNL entry points named by the
 * reference's basic/command_line.cpp:697-698 (OpenNL is an empty submodule
 * in the checkout and nothing on the kNN / convex-cell path uses it).
 * Test infrastructure for oracle/_ref only. */
#include <stdio.h>
#include "geogram/NL/nl.h"
void nlPrintfFuncs(NLprintfFunc f1, NLfprintfFunc f2) { (void)f1; (void)f2; }
void nlInitialize(int argc, char** argv) { (void)argc; (void)argv; }

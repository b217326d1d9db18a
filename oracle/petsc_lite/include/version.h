/* version.h -- stand-in for the header fvmic2d's makefile generates from its hg changeset
 * (makefile:36-37); only the options printer of io.c reads it.  TEST INFRASTRUCTURE ONLY. */
#ifndef MARKERCODE_HG_VERSION
#define MARKERCODE_HG_VERSION "oracle-build"
#endif

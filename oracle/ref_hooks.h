/* Test infrastructure (oracle only).  Force-included when the reference's
 * NC_PostProcessing.cpp is compiled for oracle/_ref/NumCalc_dump: every
 * fprintf in that file goes through oracle_fprintf, which prints floating
 * point conversions with 17 significant digits instead of the default 7.
 * The reference source itself is compiled unmodified. */
#ifndef ORACLE_REF_HOOKS_H
#define ORACLE_REF_HOOKS_H
#include <stdio.h>
#ifdef __cplusplus
/* pull in the C++ headers first: <cstdio> #undefs fprintf when included */
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
extern "C" {
#endif
int oracle_fprintf(FILE *f, const char *fmt, ...);
#ifdef __cplusplus
}
#endif
#define fprintf oracle_fprintf
#endif

/* Prototypes of the two BOINC file helpers that the reference's star reader
 * calls (milkyway_separation/cpu/star_points.c:29-38 tests `#ifdef
 * BOINC_APPLICATION`, which is true even when the macro is 0).  This header is
 * force-included (-include) into every reference translation unit so the
 * returned FILE* is not truncated to int by an implicit declaration.
 * Test infrastructure only. */
#ifndef MW_ORACLE_BOINC_SHIM_H
#define MW_ORACLE_BOINC_SHIM_H
#include <stdio.h>
#include <string.h>

int boinc_resolve_filename(const char* virtual_name, char* physical_name, int len);
FILE* boinc_fopen(const char* path, const char* mode);

#endif

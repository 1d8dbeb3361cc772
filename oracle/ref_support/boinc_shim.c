/* Host-only stand-ins for the BOINC file API: names resolve to themselves and
 * files open with fopen.  Test infrastructure only. */
#include "boinc_shim.h"

int boinc_resolve_filename(const char* virtual_name, char* physical_name, int len)
{
    if (!virtual_name || !physical_name || len <= 0)
        return 1;
    strncpy(physical_name, virtual_name, (size_t)len - 1);
    physical_name[len - 1] = '\0';
    return 0;
}

FILE* boinc_fopen(const char* path, const char* mode)
{
    return fopen(path, mode);
}

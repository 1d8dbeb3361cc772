/* Build configuration used when the reference CPU separation path is compiled
 * as a test oracle.  It stands in for the CMake-generated config.h of the
 * reference (include/config.h.in): double precision, no BOINC runtime, no
 * graphics, debug printing off.  Test infrastructure only: nothing in the
 * product links against what this builds. */
#ifndef _CONFIG_H_
#define _CONFIG_H_

#define MILKYWAY_CLIENT_VERSION_MAJOR 0
#define MILKYWAY_CLIENT_VERSION_MINOR 0
#define MILKYWAY_CLIENT_VERSION       0.0

#define BOINC_APP_VERSION "milkyway_separation_oracle 0.0"

#define DOUBLE_PRECISION 1
#define BOINC_APP_GRAPHICS 0
#define BOINC_APPLICATION 0
#define MW_DEBUG_EXCESSIVE 0

#define PRECISION "double"

#endif /* _CONFIG_H_ */

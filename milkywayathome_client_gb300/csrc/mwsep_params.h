/* mwsep_params.h -- facts about an ASTRONOMY_PARAMETERS struct shared by the
 * readers, the writers and the context. */
#ifndef MWSEP_PARAMS_H
#define MWSEP_PARAMS_H

#include "milkyway_separation_gb300.h"

/* Background values the struct holds: number_background_parameters (the
 * leading values the search maps), and at least 7 with the aux profile,
 * whose a, b, c are values 4..6 whatever number_background_parameters says
 * (init_constants, cpu/evaluation_optimized.c:72-77). */
static inline int mwsep_background_values(const ASTRONOMY_PARAMETERS* ap)
{
    const int n = ap->number_background_parameters;
    return (ap->aux_bg_profile == 1 && n < 7) ? 7 : n;
}

#endif

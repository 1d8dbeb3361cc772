/* mwsep_status.h -- status bookkeeping shared by the host sources. */
#ifndef MWSEP_STATUS_H
#define MWSEP_STATUS_H

#ifdef __cplusplus
extern "C" {
#endif
/* Record `status` as this thread's last error and return it. */
int mwsep_fail(int status);
#ifdef __cplusplus
}
#endif

#endif

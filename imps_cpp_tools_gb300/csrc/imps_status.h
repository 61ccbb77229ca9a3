// Status codes of the imps_gb300 C ABI (also declared in include/imps_gb300.h).
#pragma once

#define IMPS_OK 0
#define IMPS_WARN_NOT_CONVERGED 1
#define IMPS_ERR_BAD_ARG -1
#define IMPS_ERR_BAD_TABLE -2
#define IMPS_ERR_CUDA -3
#define IMPS_ERR_NAN -4
#define IMPS_ERR_TIMEOUT -5
#define IMPS_ERR_NO_DEVICE -6
#define IMPS_ERR_OOM -7
#define IMPS_ERR_UNSUPPORTED -8
#define IMPS_ERR_TOO_LARGE -9

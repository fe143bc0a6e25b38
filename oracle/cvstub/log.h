// log.h -- TEST INFRASTRUCTURE ONLY: silent stand-in for the reference's
// logging macros when its UCM sources are compiled as the oracle.
#ifndef GPB_CVSTUB_LOG_H
#define GPB_CVSTUB_LOG_H
#include <stdio.h>
#define log_trace(...) do { } while (0)
#define log_debug(...) do { } while (0)
#define log_info(...) do { } while (0)
#define log_warn(...) do { } while (0)
#define log_error(...) do { } while (0)
#define log_fatal(...) do { } while (0)
#endif

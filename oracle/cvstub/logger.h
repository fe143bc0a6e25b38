// logger.h -- TEST INFRASTRUCTURE ONLY: silent stand-in, see log.h.
#include "log.h"

// highgui.h -- TEST INFRASTRUCTURE ONLY: empty stand-in; cv.h holds the stub.
#include "cv.h"

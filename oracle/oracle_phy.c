// Oracle, receiver (format, demap, transform) part. TEST INFRASTRUCTURE ONLY (see oracle.h).
#include "oracle.h"

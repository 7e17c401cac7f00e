/* The reference includes matrix.h beside mex.h; everything it uses is declared in mex.h. */
#include "mex.h"

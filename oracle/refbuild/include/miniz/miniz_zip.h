/* Stand-in (see miniz.h). */
#include "miniz.h"

// Case alias: the reference includes this header under both spellings.
#include "vector3d.h"

// Case alias: the reference includes this header under both spellings.
#include "Surface.h"

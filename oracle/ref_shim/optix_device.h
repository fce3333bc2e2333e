/* TEST INFRASTRUCTURE (oracle/_ref only). */
#include "optix.h"

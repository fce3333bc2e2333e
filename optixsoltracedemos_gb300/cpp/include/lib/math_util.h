// Forwarding header: the reference addresses its headers as lib/<name>.
#include "../math_util.h"

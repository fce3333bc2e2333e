// Forwarding header: the reference addresses its headers as lib/<name>.
#include "../soltrace_system.h"

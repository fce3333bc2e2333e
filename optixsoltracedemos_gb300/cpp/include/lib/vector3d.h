// Forwarding header: the reference addresses its headers as lib/<name>.
#include "../vector3d.h"

// Forwarding header: the reference addresses its headers as lib/<name>.
#include "../element.h"

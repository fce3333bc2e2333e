/* TEST INFRASTRUCTURE (oracle/_ref only).  Force-included ahead of every reference source compiled
 * on the host: standard headers the reference sources use without including them, plus the shims. */
#ifndef ORC_REF_PRELUDE_H
#define ORC_REF_PRELUDE_H
#include <cmath>
#include <math.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cassert>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>
#include <iostream>
#include "cuda_runtime.h"
#include "optix.h"
#include "sutil/vec_math.h"
#endif

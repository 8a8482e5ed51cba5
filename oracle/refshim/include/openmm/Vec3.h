#include "../Vec3.h"

#pragma once
#include "Qhull.h"

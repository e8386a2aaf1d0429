// TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT (ds_compat; see core/Globals.h).
#pragma once
#include "Vector.h"

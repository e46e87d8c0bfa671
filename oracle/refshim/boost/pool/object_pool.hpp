// Test-only stand-in: the reference includes this header but its object_pool
// member is commented out.
#pragma once
#include "pool_alloc.hpp"

// Test-only stand-in: the reference includes this header; the call that
// used it is commented out.
#pragma once
#include <string>

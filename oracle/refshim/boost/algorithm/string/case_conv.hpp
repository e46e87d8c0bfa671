// Test-only stand-in: MuscleInterface.cpp includes this header but calls
// nothing from it.
#pragma once

// Test-only stand-in: the boost::filesystem calls the reference uses.
#pragma once
#include "boost/filesystem/operations.hpp"

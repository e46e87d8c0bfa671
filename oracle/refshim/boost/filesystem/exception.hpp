#pragma once
#include "operations.hpp"

// Test infrastructure (oracle): empty stand-in for a glm extension header.
#pragma once
#include "../glm.hpp"

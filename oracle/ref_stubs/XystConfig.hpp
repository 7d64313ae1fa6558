// Stand-in for the configure-time accessor header of the reference build.
#pragma once
#include <string>
#include "XystBuildConfig.hpp"

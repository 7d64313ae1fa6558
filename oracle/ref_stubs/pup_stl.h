// See pup.h in this folder.
#pragma once
#include "pup.h"

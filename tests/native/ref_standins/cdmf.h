// Stand-in for the reference's src/cdmf.h.
#pragma once
#include "tools.h"

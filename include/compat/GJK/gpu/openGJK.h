// GJK/gpu/openGJK.h for callers written against OpenGJK-GPU: the engine's drop-in
// declarations of the global host API (GJK/gpu/openGJK.h:91-497).
#pragma once

#include "GJK/common.h"
#include "opengjk_gpu.hpp"

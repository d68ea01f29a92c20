// Host stand-in: the launch-parameter built-ins live in cuda_runtime.h here.
#pragma once
#include "cuda_runtime.h"

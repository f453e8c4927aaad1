#pragma once
#include "cuda_shim_pre.h"

#pragma once
#include "_vtk_shim.h"

// Empty stand-in for the CUDA samples' helper_functions.h (grid.cu:7).
#pragma once

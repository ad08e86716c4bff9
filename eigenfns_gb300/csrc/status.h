// Status helpers: the last failure's detail text, kept per host thread.
#pragma once
#include <cuda_runtime.h>

int ef_fail(int code, const char* msg);
int ef_check_launch();

// every kernel launch of the library bumps this counter (ef_launch_count)
void ef_count_launches(int n);

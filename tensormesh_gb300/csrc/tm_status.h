// Status codes and the thread-local error message of the C ABI.
#pragma once
#include "../../include/tensormesh_gb300.h"

int tm_set_error(int status, const char* message);

// read and clear the PCG kernels' device fault word (1 set, 0 clear, -1 error)
int tmk_take_solve_fault();

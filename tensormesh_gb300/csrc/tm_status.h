// Status codes and the thread-local error message of the C ABI.
#pragma once
#include "../../include/tensormesh_gb300.h"

int tm_set_error(int status, const char* message);

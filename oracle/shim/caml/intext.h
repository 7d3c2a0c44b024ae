#include "poy_caml_shim.h"

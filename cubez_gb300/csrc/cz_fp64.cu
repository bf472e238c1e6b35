// Plain form: every operation in float64, as the reference (math.Real = float64).
#define CZ_R double
#define CZ_W double
#define CZ_FORM_NS fp64
#define CZ_FORM_OBJ kFormFP64
#include "cz_form_impl.cuh"

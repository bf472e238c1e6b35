// Precision form: float32 bulk arithmetic with float64 islands (quaternion
// renormalisation, adjustPositions accumulators, friction 3x3 inversion).
#define CZ_R float
#define CZ_W double
#define CZ_FORM_NS fp32
#define CZ_FORM_OBJ kFormFP32
#include "cz_form_impl.cuh"

// FP64 pixel arithmetic instantiation of the engine kernels.
#include "sa_launch_impl.cuh"
template struct sa::Launch<double>;

// trim_gb300's drop-in for the reference's umbrella header (uni10/src/uni10.hpp).
#ifndef TRIM_UNI10_HPP
#define TRIM_UNI10_HPP
#include "uni10/Qnum.h"
#include "uni10/Bond.h"
#include "uni10/Matrix.h"
#include "uni10/UniTensor.h"
#include "uni10/Network.h"
#include "uni10/Batch.h"
#endif

// Anomaly-to-anomaly Green tensor build on the device (declarations).
#pragma once

#include "egx_common.cuh"

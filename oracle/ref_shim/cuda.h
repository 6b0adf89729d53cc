/* Empty host stand-in for <cuda.h> (see cuda_runtime.h in this folder). */
#pragma once

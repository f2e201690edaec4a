/* Empty stand-in for the CUDA/OpenGL interop header that src/sim.cu:19
 * includes unconditionally; GL headers are absent and GRAPHICS is off. */
#pragma once

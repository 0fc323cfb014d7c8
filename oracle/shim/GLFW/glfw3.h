// Project-written headless stand-in: the reference's Shader.h includes the
// windowing header, but nothing on the CPU solver path calls into it.
// Test infrastructure only.
#ifndef NBODY_SHIM_GLFW3_H
#define NBODY_SHIM_GLFW3_H
#endif

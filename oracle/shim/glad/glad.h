// Project-written headless stand-in for the OpenGL loader header. It declares
// only the GL types, enums and buffer entry points that the reference's CPU
// solver path touches (persistently mapped buffers in ParticleSystem and the
// OpenGLBuffer wrapper). The definitions in gl_stub.cpp keep every buffer in
// plain host memory; no graphics API is brought up and no shader ever runs.
// Test infrastructure only.
#ifndef NBODY_SHIM_GLAD_H
#define NBODY_SHIM_GLAD_H

#include <cstddef>
#include <cstdint>

typedef unsigned int GLenum;
typedef unsigned int GLuint;
typedef int GLint;
typedef int GLsizei;
typedef unsigned int GLbitfield;
typedef unsigned char GLboolean;
typedef float GLfloat;
typedef char GLchar;
typedef std::ptrdiff_t GLsizeiptr;
typedef std::ptrdiff_t GLintptr;

#define GL_FALSE 0
#define GL_TRUE 1
#define GL_NO_ERROR 0
#define GL_SHADER_STORAGE_BUFFER 0x90D2
#define GL_DYNAMIC_COPY 0x88EA
#define GL_STATIC_DRAW 0x88E4
#define GL_MAP_READ_BIT 0x0001
#define GL_MAP_WRITE_BIT 0x0002
#define GL_MAP_PERSISTENT_BIT 0x0040
#define GL_MAP_COHERENT_BIT 0x0080
#define GL_SHADER_STORAGE_BARRIER_BIT 0x00002000
#define GL_COMPUTE_SHADER 0x91B9
#define GL_VERTEX_SHADER 0x8B31
#define GL_FRAGMENT_SHADER 0x8B30
#define GL_COMPILE_STATUS 0x8B81
#define GL_LINK_STATUS 0x8B82

void glGenBuffers(GLsizei n, GLuint *buffers);
void glDeleteBuffers(GLsizei n, const GLuint *buffers);
void glBindBuffer(GLenum target, GLuint buffer);
void glBindBufferBase(GLenum target, GLuint index, GLuint buffer);
void glBufferStorage(GLenum target, GLsizeiptr size, const void *data, GLbitfield flags);
void glBufferData(GLenum target, GLsizeiptr size, const void *data, GLenum usage);
void glBufferSubData(GLenum target, GLintptr offset, GLsizeiptr size, const void *data);
void glGetBufferSubData(GLenum target, GLintptr offset, GLsizeiptr size, void *data);
void *glMapBufferRange(GLenum target, GLintptr offset, GLsizeiptr length, GLbitfield access);
GLboolean glUnmapBuffer(GLenum target);
GLenum glGetError(void);
void glDispatchCompute(GLuint x, GLuint y, GLuint z);
void glMemoryBarrier(GLbitfield barriers);

#endif

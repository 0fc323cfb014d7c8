// Headless link-level stand-ins for the graphics calls that the reference's CPU
// solver path reaches (ParticleSystem's persistently mapped buffers, the
// OpenGLBuffer wrapper and the Shader constructors it triggers). Buffers are
// plain host allocations; mapping returns that memory; shader compilation and
// dispatch are no-ops. No graphics API is brought up and no shader source is
// read or run. Test infrastructure only: linked into oracle/_ref, never into
// the product.
#include <glad/glad.h>

#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "ComputeShader.h"
#include "Shader.h"

namespace {
struct HostBuffer {
    std::vector<unsigned char> bytes;
};
std::mutex g_mu;
std::map<GLuint, HostBuffer> g_buffers;
GLuint g_next_id = 1;
GLuint g_bound = 0;
}  // namespace

void glGenBuffers(GLsizei n, GLuint *buffers) {
    std::lock_guard<std::mutex> lk(g_mu);
    for (GLsizei i = 0; i < n; ++i) {
        buffers[i] = g_next_id++;
        g_buffers[buffers[i]];
    }
}

void glDeleteBuffers(GLsizei n, const GLuint *buffers) {
    std::lock_guard<std::mutex> lk(g_mu);
    for (GLsizei i = 0; i < n; ++i) g_buffers.erase(buffers[i]);
}

void glBindBuffer(GLenum, GLuint buffer) { g_bound = buffer; }
void glBindBufferBase(GLenum, GLuint, GLuint) {}

static void store(GLsizeiptr size, const void *data) {
    std::lock_guard<std::mutex> lk(g_mu);
    HostBuffer &b = g_buffers[g_bound];
    b.bytes.assign(static_cast<size_t>(size), 0);
    if (data) std::memcpy(b.bytes.data(), data, static_cast<size_t>(size));
}

void glBufferStorage(GLenum, GLsizeiptr size, const void *data, GLbitfield) { store(size, data); }
void glBufferData(GLenum, GLsizeiptr size, const void *data, GLenum) { store(size, data); }

void glBufferSubData(GLenum, GLintptr offset, GLsizeiptr size, const void *data) {
    std::lock_guard<std::mutex> lk(g_mu);
    std::memcpy(g_buffers[g_bound].bytes.data() + offset, data, static_cast<size_t>(size));
}

void glGetBufferSubData(GLenum, GLintptr offset, GLsizeiptr size, void *data) {
    std::lock_guard<std::mutex> lk(g_mu);
    std::memcpy(data, g_buffers[g_bound].bytes.data() + offset, static_cast<size_t>(size));
}

void *glMapBufferRange(GLenum, GLintptr offset, GLsizeiptr, GLbitfield) {
    std::lock_guard<std::mutex> lk(g_mu);
    return g_buffers[g_bound].bytes.data() + offset;
}

GLboolean glUnmapBuffer(GLenum) { return GL_TRUE; }
GLenum glGetError(void) { return GL_NO_ERROR; }
void glDispatchCompute(GLuint, GLuint, GLuint) {}
void glMemoryBarrier(GLbitfield) {}

// Shader objects: the CPU path constructs three of them in ParticleSystem's
// constructor but never dispatches them, so the stand-ins hold no state.
Shader::Shader() = default;
Shader::~Shader() = default;
void Shader::use() const {}
void Shader::setBool(const std::string &, bool) const {}
void Shader::setInt(const std::string &, int) const {}
void Shader::setFloat(const std::string &, float) const {}
void Shader::setVec2(const std::string &, const glm::vec2 &) const {}
void Shader::setVec2(const std::string &, float, float) const {}
void Shader::setVec3(const std::string &, const glm::vec3 &) const {}
void Shader::setVec3(const std::string &, float, float, float) const {}
void Shader::setVec4(const std::string &, const glm::vec4 &) const {}
void Shader::setVec4(const std::string &, float, float, float, float) const {}
void Shader::setMat2(const std::string &, const glm::mat2 &) const {}
void Shader::setMat3(const std::string &, const glm::mat3 &) const {}
void Shader::setMat4(const std::string &, const glm::mat4 &) const {}
void Shader::checkCompileErrors(unsigned int, std::string) {}
unsigned int Shader::compileShader(GLuint, const char *) { return 0; }
std::string Shader::readFileToString(const std::string &) { return std::string(); }
ComputeShader::ComputeShader(const std::string &) : Shader() { ID = 0; }

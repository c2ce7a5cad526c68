// Type-only stand-in for GLEW (test infrastructure: lets the reference headers
// that mention GL handle types compile; no GL function is ever declared or called).
#pragma once
typedef unsigned int GLuint;
typedef int GLint;
typedef unsigned int GLenum;
typedef float GLfloat;
typedef int GLsizei;
typedef unsigned char GLboolean;
typedef void GLvoid;

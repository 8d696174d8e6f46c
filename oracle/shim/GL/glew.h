/* Headless stand-in for the GL loader header, used only when oracle/Makefile compiles the
 * reference's physics sources for the oracle. src/entity.cpp includes <GL/glew.h> for
 * entity_mesh_replace, which the physics path never calls; these two no-op declarations are all
 * that translation unit needs. */
#ifndef RP_ORACLE_HEADLESS_GLEW_H
#define RP_ORACLE_HEADLESS_GLEW_H
static inline void glDeleteBuffers(int n, const unsigned int* names) { (void)n; (void)names; }
static inline void glDeleteVertexArrays(int n, const unsigned int* names) { (void)n; (void)names; }
#endif

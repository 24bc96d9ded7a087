/* Stand-in for <GL/glu.h>: see GL/gl.h in this directory. */
#ifndef MILTON_REF_SHIM_GLU_H_
#define MILTON_REF_SHIM_GLU_H_
#include <GL/gl.h>
typedef struct GLUquadric GLUquadric;
typedef GLUquadric GLUquadricObj;
static inline void gluDeleteQuadric(GLUquadric *) {}
static inline GLUquadric *gluNewQuadric(void) { return 0; }
static inline const unsigned char *gluErrorString(GLenum) { return (const unsigned char *)""; }
static inline void gluSphere(GLUquadric *, GLdouble, GLint, GLint) {}
static inline void gluQuadricNormals(GLUquadric *, GLenum) {}
static inline void gluQuadricTexture(GLUquadric *, GLboolean) {}
static inline void gluCylinder(GLUquadric *, GLdouble, GLdouble, GLdouble, GLint, GLint) {}
static inline void gluDisk(GLUquadric *, GLdouble, GLdouble, GLint, GLint) {}
#endif

/* oldefine.h (drop-in) -- enums of the reference's include/oldefine.h:7-13
 * (and ol::INTERPOLATION, olprop.h:408-410). */
#ifndef OLGB300_OLDEFINE_H
#define OLGB300_OLDEFINE_H
#define F32_PI 3.14159265f
namespace ol {
enum PROPMODE { ASM, FRESNEL, AUTO };
enum HOLOGRAMSTEP { RECORD, PLAY };
enum MODE { PHASE, REAL, IMAG, AMP };
// olprop.h:408-410
enum INTERPOLATION { BILINEAR, BICUBIC };
} // namespace ol
#endif

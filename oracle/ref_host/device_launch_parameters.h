// Host build of the reference renderer: thread/block indices are declared by
// isti_refhost.h (force-included), so the CUDA header of this name is shadowed.
#pragma once

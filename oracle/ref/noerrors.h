/* Empty stand-in for the reference kernels' noerrors.h, which only exists to pull host declarations into an IDE. */
#pragma once

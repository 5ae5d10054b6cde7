/* The reference includes this header; its sparse BLAS calls are commented out. */
#pragma once

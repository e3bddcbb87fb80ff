// 2D-velocity operator in FP64: dispatch on the grid size.
#include "collide2d.cuh"

namespace pii {

int collide2d_f64(pii_plan* p, const double* f, double* q, int64_t cells, int with_loss, double hb,
                   cudaStream_t s) {
  switch (p->n) {
    case 8: return Collide2D<double, 8>::run(p, f, q, cells, with_loss, hb, s);
    case 16: return Collide2D<double, 16>::run(p, f, q, cells, with_loss, hb, s);
    case 24: return Collide2D<double, 24>::run(p, f, q, cells, with_loss, hb, s);
    case 32: return Collide2D<double, 32>::run(p, f, q, cells, with_loss, hb, s);
    case 48: return Collide2D<double, 48>::run(p, f, q, cells, with_loss, hb, s);
    case 64: return Collide2D<double, 64>::run(p, f, q, cells, with_loss, hb, s);
    default: set_error("collide (2D): unsupported n = %d", p->n); return PII_ERR_ARG;
  }
}

int laplacian2d_f64(pii_plan* p, const double* f, double* out, int64_t cells, cudaStream_t s) {
  switch (p->n) {
    case 8: return Collide2D<double, 8>::laplacian(p, f, out, cells, s);
    case 16: return Collide2D<double, 16>::laplacian(p, f, out, cells, s);
    case 24: return Collide2D<double, 24>::laplacian(p, f, out, cells, s);
    case 32: return Collide2D<double, 32>::laplacian(p, f, out, cells, s);
    case 48: return Collide2D<double, 48>::laplacian(p, f, out, cells, s);
    case 64: return Collide2D<double, 64>::laplacian(p, f, out, cells, s);
    default: set_error("laplacian (2D): unsupported n = %d", p->n); return PII_ERR_ARG;
  }
}

}  // namespace pii

// engine_types.hh -- device-visible data layout of the gbint engine.
//
// Every integrator family of the reference is a tensor product of at most four quadrature
// axes.  The host turns each axis into a node array (value, weight) with the reference's
// maps and Jacobians folded in (x -> q = k sqrt(x x_extent), cos = 2(t-1/2), phi = 2 pi t,
// int_element, Matsubara or explicit-sum weights), so the device evaluates
//     constant + sum_{i0..i3} w0[i0] w1[i1] w2[i2] w3[i3] * KERNEL(v0[i0], v1[i1], ...)
// with every "q0" axis evaluated at +-v (nodes before pm_from are evaluated once).
#pragma once

#include <cstdint>

#include "gbint.h"
#include "gbint/device/numerics.cuh"

namespace gbint
{
  // coordinate an axis feeds into the kernel
  enum Role : int { R_NONE = 0, R_Q = 1, R_C1 = 2, R_C2 = 3, R_PHI = 4, R_Q0 = 5, R_QX = 6, R_QY = 7, R_QZ = 8 };

  // 32-byte node record for FP32 kernels, every field a double-float pair:
  // v = coordinate, w = weight, a = auxiliary value (sqrt(1 - v^2) on cos axes, cos(v) on phi
  // axes, v^2 on radial axes), aw = w * a.
  struct alignas(32) NodeRec {
    float v_hi, v_lo, w_hi, w_lo, a_hi, a_lo, aw_hi, aw_lo;
  };

  struct AxisRef {
    int off;      // node index into the pools
    int n;        // nodes
    int role;     // Role
    int pm_from;  // nodes >= pm_from are evaluated at +v and -v
  };

  // kernel kinds
  enum Kind : int {
    K_GENERIC = 0,  // any family x any integrand, FP64, thread per point
    K_S1 = 1,       // 2-axis (q, c) + PROP1, FP32c: rows q, inner c
    K_S2 = 2,       // (mode, q, c) + FTLOOP, FP32c: rows (mode, q), inner c
    K_S3 = 3,       // (q, c, phi) + PROP3, FP32c: rows (q, c), inner phi
    K_S5 = 5,       // (q, c1, c2, phi) + VERT4, FP32c: rows (q, c1), mid c2, inner phi
    K_S5Z = 6,      // K_S5, accurate form only, with the 2D tables read through slices along their
                    // cos axis (rows ordered (c1, q); chosen when the slices fit shared memory)
    K_S3R = 7,      // K_S3, accurate form only, with the three point-dependent tables read through
                    // their per-cell records (chosen when all three carry records)
    K_ACC = 16      // flag on K_S*: double-float evaluation of the per-point factors
  };
  constexpr int kind_base(int k) { return k & 15; }
  constexpr bool kind_acc(int k) { return (k & K_ACC) != 0; }

  struct ItemDev {
    int kind;
    int integrand;
    int family;
    int n_axes;
    int rows;        // rows (S kinds) or points (generic)
    AxisRef ax[4];
    int unit_begin;
    int n_units;
    int seg_off;     // hoisted FP64 factors (S kinds)
    int seg_stride;  // row stride inside the segment
    int tab[4];      // table directory slots
    int aux_off;     // per-item constants of the S kinds in RunParams::aux (float4 records)
    int slice_off;   // S2 (accurate form): mode-interpolated table slices in the segment arena (doubles);
                     // S5Z: table A at the c1 nodes
    int slice_off2;  // S5Z: table B at the c2 nodes
    int slice_off3;  // S5Z: table A at the c2 nodes
    int split_log2;  // S3 / S5Z: each quadrature row is split into 2^split_log2 parts of its inner
                     // (S3: phi) or middle (S5Z: c2) loop; rows counts the parts
    double k;
    double args[GB_MAX_ARGS];
  };

  struct UnitDev {
    int item;
    int row_begin;
    int row_count;
    int slot;  // partial-sum slot: the unit's position in item order (units may run in another order)
  };

  // the work units of one integral, expanded on the device into UnitDev records
  // (units[unit0 + u] = {item, u * rpu, min(rpu, rows - u * rpu), slot0 + u}): the host plans
  // per integral, not per unit
  struct ExpandDev {
    int item, unit0, n_units, rows, rpu, slot0;
  };

  // table directory entry (device): current FP32 data + axes
  struct TableDev {
    const float *data;
    int n0, n1;  // n1 == 0: 1D
    int bytes;   // bytes staged per table (data, then the cell-centre reciprocals), multiple of 16
    int rc_off;   // float offset of the (hi, lo) reciprocals of the cell centres of axis rc_axis; 0: none
    int rc_axis;  // the log axis they belong to (cells at most 25 % wide)
    int rc_sq;    // 1: cells at most 12 % wide, so the reciprocals also serve a squared coordinate
    int rq_off;   // float offset of the regulator's per-cell Taylor coefficients (global only); 0: none
    int cr_off;   // float offset of the per-cell value records (1D log tables with reciprocals; 0:
                  // none): float4 {1/c_j hi, 1/c_j lo, y_j, hi(y_{j+1} - y_j)} per cell, then per
                  // cell the low word of the difference (y_{j+1} - y_j = hi + lo exactly), rebuilt
                  // on update
    int gr_off;   // float offset of the per-cell propagator records (with rq_off; 0: none), four
                  // float4 arrays of a float4 per cell, rebuilt on update: {1/c_j hi, lo, g0 hi, lo}, {g1 hi, lo, g2 hi,
                  // lo}, {g3, g4, g5, g6}, {g7, g8, el, +-eh} -- 1 / (Z(x) x + R(x)) = sum g_k t^k
                  // through t^8, t = x / c_j - 1; (el, eh) the cell's edges in t moved inwards by
                  // 4e-7; eh < 0: the series was not trusted over the cell
    int rd_off;   // float offset of the regulator's per-cell Taylor coefficients in FP64 (10 a
                  // cell; with gr_off), read only when the records are built
    double e_lo, e_hi;  // with cr_off: the edges of every cell in t = x / c_j - 1, 2^(-+1/(2 scale)) - 1
    dev::AxisDev a0, a1;
  };

  constexpr int kMaxTables = 256;

  // bits of the context's device error word (RunParams::err)
  constexpr int kErrMbarTimeout = 1;  // a bounded mbarrier wait gave up
  constexpr int kErrBadIndex = 2;     // a work unit or table index out of range was skipped

  struct RunParams {
    const ItemDev *items;
    const UnitDev *units;
    int n_units;
    int n_items;
    const double *pv;      // FP64 node values
    const double *pw;      // FP64 node weights
    const double *pa;      // FP64 aux values
    const NodeRec *prec;   // FP32 records
    const TableDev *tabs;  // directory
    const double *seg;     // hoisted factors
    const float4 *aux;     // per-item double-float constants and S2 mode records
    double *partials;      // per unit
    int *item_count;       // per item arrival counters (reset by the finisher)
    int *unit_counter;     // work-stealing counter (reset by the finisher of the run)
    int single;            // 1: CTA b evaluates unit b only and retires (a grid of one CTA per
                           // unit), so that CTAs of a later high-priority launch get SMs as soon
                           // as units finish; 0: persistent CTAs take units from unit_counter
    int *done_counter;     // items finished in this run
    double *out;           // per item results
    int *err;              // device error word
  };

  // hoisted-factor segment kinds
  // SEG_S2Z: the S2 dressing table interpolated along its mode axis at every (mode, sign)
  // frequency of an item, per |q| cell: float4 {z hi, lo, dz hi, lo} (two doubles per entry)
  // SEG_AX1: a 2D table interpolated along its second axis at the nodes of a quadrature axis,
  // per first-axis cell: float4 {z hi, lo, dz hi, lo}
  enum SegKind : int { SEG_S1 = 1, SEG_S2 = 2, SEG_S3 = 3, SEG_S5 = 5, SEG_S2Z = 6, SEG_AX1 = 7 };
  struct SegDev {
    int kind;
    int off;       // output offset
    int n0, n1;    // entries = n0 * n1
    AxisRef ax0, ax1;
    int tab;       // table slot
    int aux_off;   // SEG_S2: per-q FP64 factors in RunParams::aux (3 float4 = 6 doubles per q node)
    double par[4];
  };
} // namespace gbint

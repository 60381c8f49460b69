// Many independent solves (snapshots of uneven size) as one device program.
//
// The reference images a list of visibility blocks with one Dask task per
// block (rascil/workflows/rsexecute/imaging/imaging_rsexecute.py:72-157);
// here a list of plans is one program of rounds.  Plan i is bound to
// workspace slot i % nslots; a slot runs its plans in order (bucket sort,
// invert over its batches of w-planes, predict over them), and every round
// takes the next batch of w-planes of every slot's current plan as a job:
//
//   fork     each slot's stream waits for the main stream, then runs its
//            own steps: a new plan's bucket sort and per-item values, the
//            zeroing of an invert batch, or the screens and transforms of a
//            predict batch;
//   join     the main stream waits for every slot;
//   grid     ONE persistent k_grid_jobs launch per (pols, lane width) grids
//            every invert job's chunks, fed from a device work queue (the
//            jobs' chunk ranges concatenated, one atomic counter);
//   degrid   ONE persistent k_degrid_warp_jobs launch per (pols, lane width)
//            degrids every predict job's chunks the same way;
//   fork     each invert job's transforms, screens and image accumulation
//            (and its plan's correction pass after the last batch) run on
//            its slot's stream.
//
// Small snapshots, whose own launches would leave most of the GPU idle,
// share the gridding and degridding launches of every round with the large
// ones; the transforms of different slots overlap on their streams.  Every
// step is a stream operation, so the whole program can be captured in a
// CUDA graph.  FP64-form plans run their calls per plan on the slot
// streams.
#include <cstring>
#include <vector>

#include "gb_fft.cuh"
#include "gb_plan.cuh"

using namespace gb;

namespace {

enum Phase { kBind = 0, kInvert, kPredict, kDone };

struct Slot {
  std::vector<int> plans;  // indices into the batch, in order
  size_t next = 0;         // next plan to take
  int cur = -1;            // current plan index, -1 = none
  Phase phase = kBind;
  int bi = 0;              // next w-plane batch of the phase
  cudaStream_t s = nullptr;
  cudaEvent_t ev = nullptr;
  bool grid_job = false, degrid_job = false;
};

struct Args {  // one solve's arguments, validated, matrices built
  gb_batch_item it;
  PolMat pm_in, pm_out;
  bool inv, pred;
};

bool same_pm(const PolMat &a, const PolMat &b) {
  if (a.identity && b.identity) return a.nout == b.nout;
  return a.identity == b.identity && a.nout == b.nout && a.nin == b.nin &&
         memcmp(a.re, b.re, sizeof(a.re)) == 0 && memcmp(a.im, b.im, sizeof(a.im)) == 0;
}

int run_items(gb_plan *const *plans, const gb_batch_item *items, int32_t nplans,
              void *const *workspaces, const size_t *workspace_bytes, void *const *streams,
              int32_t nslots, int32_t layout) {
  if (nplans < 0 || (nplans > 0 && (!plans || !items || !workspaces || !workspace_bytes ||
                                    !streams)) ||
      nslots < 1 || nslots > kMaxJobs) {
    set_error("gb_batch_run: NULL array, or nslots outside 1..%d", kMaxJobs);
    return GB_ERR_INVALID_ARG;
  }
  if (layout != GB_LAYOUT_XY && layout != GB_LAYOUT_YX) {
    set_error("gb_batch_run: unknown layout %d", layout);
    return GB_ERR_INVALID_ARG;
  }
  std::vector<Args> args(nplans);
  for (int32_t i = 0; i < nplans; ++i) {
    gb_plan *p = plans[i];
    Args &a = args[i];
    a.it = items[i];
    if (!p) {
      set_error("gb_batch_run: plan %d is NULL", (int)i);
      return GB_ERR_INVALID_ARG;
    }
    a.inv = a.it.vis || a.it.psf;
    a.pred = a.it.model != nullptr;
    const int np = p->g.NP;
    if (a.inv) {
      if (!a.it.dirty) {
        set_error("gb_batch_run: plan %d has visibilities but no dirty image", (int)i);
        return GB_ERR_INVALID_ARG;
      }
      if (a.it.npol_vis < np || a.it.npol_vis > 4) {
        set_error("gb_batch_run: plan %d: npol_vis %d outside [npol=%d, 4]", (int)i,
                  a.it.npol_vis, np);
        return GB_ERR_INVALID_ARG;
      }
      if (!a.it.flags) a.it.flags_type = GB_FLAGS_NONE;
      if (a.it.flags && a.it.flags_type != GB_FLAGS_U8 && a.it.flags_type != GB_FLAGS_I64) {
        set_error("gb_batch_run: plan %d: flags_type %d unknown", (int)i, a.it.flags_type);
        return GB_ERR_INVALID_ARG;
      }
      const int rc = make_polmat(a.it.polmat_in, np, a.it.npol_vis, a.pm_in);
      if (rc) return rc;
    }
    if (a.pred) {
      if (!a.it.pred) {
        set_error("gb_batch_run: plan %d has a model but no output visibilities", (int)i);
        return GB_ERR_INVALID_ARG;
      }
      if (a.it.npol_out < np || a.it.npol_out > 4) {
        set_error("gb_batch_run: plan %d: npol_out %d outside [npol=%d, 4]", (int)i,
                  a.it.npol_out, np);
        return GB_ERR_INVALID_ARG;
      }
      const int rc = make_polmat(a.it.polmat_out, a.it.npol_out, np, a.pm_out);
      if (rc) return rc;
    }
    if (workspace_bytes[i % nslots] < p->ws_bytes) {
      set_error("gb_batch_run: workspace %d holds %zu bytes, plan %d needs %zu", (int)(i % nslots),
                workspace_bytes[i % nslots], (int)i, p->ws_bytes);
      return GB_ERR_WORKSPACE;
    }
  }
  if (nplans == 0) return GB_OK;
  int dev = 0, sms = 0;
  GB_CUDA(cudaGetDevice(&dev));
  GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  cudaStream_t main = (cudaStream_t)streams[0];
  std::vector<Slot> slots(nslots);
  for (int k = 0; k < nslots; ++k) {
    slots[k].s = (cudaStream_t)streams[k];
    for (int i = k; i < nplans; i += nslots) slots[k].plans.push_back(i);
  }
  cudaEvent_t ev_main = nullptr;
  int rc = GB_OK;
#define GB_TRY(call)      \
  do {                    \
    const int r__ = (call); \
    if (r__) {            \
      rc = r__;           \
      goto done;          \
    }                     \
  } while (0)
#define GB_TRYC(call) \
  GB_TRY(((call) == cudaSuccess) ? GB_OK : cuda_fail(cudaGetLastError(), #call))
  GB_TRYC(cudaEventCreateWithFlags(&ev_main, cudaEventDisableTiming));
  for (auto &sl : slots) GB_TRYC(cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming));
  for (;;) {
    // fork: every slot's own steps up to its next job
    GB_TRYC(cudaEventRecord(ev_main, main));
    bool any = false;
    for (int k = 0; k < nslots; ++k) {
      Slot &sl = slots[k];
      sl.grid_job = sl.degrid_job = false;
      if (sl.cur < 0 && sl.next >= sl.plans.size()) continue;
      GB_TRYC(cudaStreamWaitEvent(sl.s, ev_main, 0));
      for (;;) {
        if (sl.cur < 0 || sl.phase == kDone) {
          if (sl.next >= sl.plans.size()) {
            sl.cur = -1;
            break;
          }
          sl.cur = sl.plans[sl.next++];
          sl.phase = kBind;
        }
        const int i = sl.cur;
        gb_plan *p = plans[i];
        const Args &a = args[i];
        if (sl.phase == kBind) {
          GB_TRY(gb_plan_bind(p, workspaces[k], workspace_bytes[k], sl.s));
          sl.bi = 0;
          if (p->precision == GB_FP64) {  // the FP64 form: whole calls per plan
            if (a.inv)
              GB_TRY(run_ms2dirty(p, a.it.vis, a.it.npol_vis, a.it.wgt, a.it.flags,
                                  a.it.flags_type, a.pm_in, a.it.psf, a.it.dirty, layout,
                                  a.it.sumwt, sl.s));
            if (a.pred)
              GB_TRY(run_dirty2ms(p, a.it.model, layout, nullptr, a.pm_out, a.it.npol_out,
                                  a.it.pred, sl.s));
            sl.phase = kDone;
            continue;
          }
          if (a.inv) {
            GB_TRY(inv_begin(p, a.it.vis, a.it.npol_vis, a.it.wgt, a.it.flags, a.it.flags_type,
                             a.pm_in, a.it.psf, a.it.sumwt, sl.s));
            sl.phase = kInvert;
          } else if (a.pred) {
            GB_TRY(pred_begin(p, a.it.model, layout, sl.s));
            sl.phase = kPredict;
          } else {
            sl.phase = kDone;
            continue;
          }
        }
        if (sl.phase == kInvert) {
          GB_TRY(inv_zero(p, sl.bi, sl.s));
          sl.grid_job = true;
        } else {
          GB_TRY(pred_transform(p, sl.bi, sl.s));
          sl.degrid_job = true;
        }
        break;
      }
      if (sl.grid_job || sl.degrid_job) any = true;
      // join
      GB_TRYC(cudaEventRecord(sl.ev, sl.s));
      GB_TRYC(cudaStreamWaitEvent(main, sl.ev, 0));
    }
    if (!any) break;
    // the round's persistent launches on the main stream, one per group
    for (int pass = 0; pass < 2; ++pass) {
      std::vector<bool> taken(nslots, false);
      for (int k0 = 0; k0 < nslots; ++k0) {
        const bool want0 = pass == 0 ? slots[k0].grid_job : slots[k0].degrid_job;
        if (!want0 || taken[k0]) continue;
        const int i0 = slots[k0].cur;
        gb_plan *p0 = plans[i0];
        GridJobs jobs;
        jobs.n = 0;
        double bytes = 0.0, updates = 0.0;
        for (int k = k0; k < nslots; ++k) {
          Slot &sl = slots[k];
          const bool want = pass == 0 ? sl.grid_job : sl.degrid_job;
          if (!want || taken[k]) continue;
          gb_plan *p = plans[sl.cur];
          const bool same =
              p->g.NP == p0->g.NP &&
              (pass == 0 ? group_lanes(p->g.W) == group_lanes(p0->g.W)
                         : p->g.W == p0->g.W && same_pm(args[sl.cur].pm_out, args[i0].pm_out));
          if (!same) continue;
          taken[k] = true;
          double b = 0.0, u = 0.0;
          if (pass == 0) {
            GB_TRY(grid_job(p, sl.bi, jobs.job[jobs.n]));
            grid_job_counts(p, sl.bi, &b, &u);
          } else {
            const Args &a = args[sl.cur];
            GB_TRY(degrid_job(p, sl.bi, a.it.pred, a.it.npol_out, jobs.job[jobs.n]));
            degrid_job_counts(p, sl.bi, a.it.npol_out, &b, &u);
          }
          bytes += b;
          updates += u;
          ++jobs.n;
        }
        // the first job's per-batch counter was zeroed by its plan's begin step
        uint32_t *counter = p0->at<uint32_t>(p0->off_counters) + (pass == 0 ? 0 : p0->nbatches) +
                            slots[k0].bi;
        if (pass == 0)
          GB_TRY(launch_grid_jobs(jobs, sms, counter, bytes, updates, main));
        else
          GB_TRY(launch_degrid_jobs(jobs, args[i0].pm_out, sms, counter, bytes, updates, main));
      }
    }
    // fork: the invert jobs' transforms; advance every slot
    GB_TRYC(cudaEventRecord(ev_main, main));
    for (int k = 0; k < nslots; ++k) {
      Slot &sl = slots[k];
      if (!sl.grid_job && !sl.degrid_job) continue;
      const int i = sl.cur;
      gb_plan *p = plans[i];
      const Args &a = args[i];
      if (sl.grid_job) {
        GB_TRYC(cudaStreamWaitEvent(sl.s, ev_main, 0));
        GB_TRY(inv_transform(p, sl.bi, sl.s));
        if (++sl.bi == p->nbatches) {
          GB_TRY(inv_end(p, a.it.dirty, layout, sl.s));
          sl.bi = 0;
          if (a.pred) {
            GB_TRY(pred_begin(p, a.it.model, layout, sl.s));
            sl.phase = kPredict;
          } else {
            sl.phase = kDone;
          }
        }
      } else if (++sl.bi == p->nbatches) {
        sl.phase = kDone;
      }
    }
  }
  // the main stream ends after every slot's last step
  for (auto &sl : slots) {
    GB_TRYC(cudaEventRecord(sl.ev, sl.s));
    GB_TRYC(cudaStreamWaitEvent(main, sl.ev, 0));
  }
done:
  for (auto &sl : slots)
    if (sl.ev) cudaEventDestroy(sl.ev);
  if (ev_main) cudaEventDestroy(ev_main);
#undef GB_TRYC
#undef GB_TRY
  return rc;
}

}  // namespace

extern "C" {

int gb_batch_run_items(gb_plan *const *plans, const gb_batch_item *items, int32_t nplans,
                       void *const *workspaces, const size_t *workspace_bytes,
                       void *const *streams, int32_t nslots, int32_t layout) {
  return run_items(plans, items, nplans, workspaces, workspace_bytes, streams, nslots, layout);
}

int gb_batch_run(gb_plan *const *plans, int32_t nplans, void *const *workspaces,
                 const size_t *workspace_bytes, void *const *streams, int32_t nslots,
                 const void *const *vis, void *const *dirty, const void *const *model,
                 void *const *pred, int32_t layout) {
  if (nplans < 0 || (nplans > 0 && !plans)) {
    set_error("gb_batch_run: NULL plans");
    return GB_ERR_INVALID_ARG;
  }
  std::vector<gb_batch_item> items(nplans > 0 ? nplans : 0);
  for (int32_t i = 0; i < nplans; ++i) {
    gb_batch_item &it = items[i];
    memset(&it, 0, sizeof(it));
    const int np = plans[i] ? plans[i]->g.NP : 1;
    it.vis = vis ? vis[i] : nullptr;
    it.npol_vis = np;
    it.dirty = dirty ? dirty[i] : nullptr;
    it.model = model ? model[i] : nullptr;
    it.npol_out = np;
    it.pred = pred ? pred[i] : nullptr;
    if (it.vis && !it.dirty) {
      set_error("gb_batch_run: plan %d has visibilities but no dirty image", (int)i);
      return GB_ERR_INVALID_ARG;
    }
  }
  return run_items(plans, items.data(), nplans, workspaces, workspace_bytes, streams, nslots,
                   layout);
}

}  // extern "C"

// Full-state checkpoints for an exact restart (owt_checkpoint_*) and the
// device-kept state (owt_state_keep / owt_state_restore).
#include "handle.h"

using namespace owt;

extern "C" {

// Checkpoint image: header, then fields in level order (independent of the
// ring slots), then the NY-vectors and scalars.
namespace {
struct CkptHeader {
  char magic[8];
  int64_t version, NX, NY, NZ, step, precision;
  double dt, dkx, dkz, alpha_mesh, nu;
};
const int kRings = 5, kFields = 7;
}  // namespace

int owt_checkpoint_bytes(const owt_handle *h, int64_t *bytes) {
  if (!h || !bytes) return OWT_ERR_INVALID;
  const size_t f = h->fs * sizeof(double2), v = (size_t)h->NY * sizeof(double2);
  *bytes = (int64_t)(sizeof(CkptHeader) + (3 * kRings + kFields) * f + 12 * v + 6 * sizeof(double));
  return OWT_OK;
}

int owt_checkpoint_save(owt_handle *h, void *host, int64_t bytes) {
  return guard(h, [&] {
    int64_t need = 0;
    owt_checkpoint_bytes(h, &need);
    if (!host || bytes < need) throw OwtError(OWT_ERR_INVALID, "checkpoint buffer too small");
    ck(cudaStreamSynchronize(h->st), "checkpoint");
    h->recompute_dirty_q();
    CkptHeader hd{};
    std::memcpy(hd.magic, "OWTCKPT1", 8);
    hd.version = 1; hd.NX = h->NX; hd.NY = h->NY; hd.NZ = h->NZ; hd.step = h->steps; hd.precision = h->precision;
    hd.dt = h->p.dt; hd.dkx = h->p.dkx; hd.dkz = h->p.dkz; hd.alpha_mesh = h->p.alpha_mesh; hd.nu = h->p.nu;
    char *o = static_cast<char *>(host);
    std::memcpy(o, &hd, sizeof(hd));
    o += sizeof(hd);
    const size_t f = h->fs * sizeof(double2), v = (size_t)h->NY * sizeof(double2);
    for (double2 *ring : {h->v_ring, h->g_ring, h->hv_ring, h->hg_ring, h->q_ring})
      for (int l = 0; l < 3; ++l, o += f)
        ck(cudaMemcpyAsync(o, h->ring_level(ring, l), f, cudaMemcpyDeviceToHost, h->st), "D2H");
    for (double2 *fld : {h->u, h->w, h->ox, h->oz, h->lx, h->ly, h->lz}) {
      ck(cudaMemcpyAsync(o, fld, f, cudaMemcpyDeviceToHost, h->st), "D2H");
      o += f;
    }
    for (double2 *ring : {h->lxm_ring, h->lzm_ring, h->U_ring, h->W_ring})
      for (int l = 0; l < 3; ++l, o += v)
        ck(cudaMemcpyAsync(o, ring + (size_t)h->slot(l) * h->NY, v, cudaMemcpyDeviceToHost, h->st), "D2H");
    for (double *fr : {h->fx_ring, h->fz_ring})
      for (int l = 0; l < 3; ++l, o += sizeof(double))
        ck(cudaMemcpyAsync(o, fr + h->slot(l), sizeof(double), cudaMemcpyDeviceToHost, h->st), "D2H");
    ck(cudaStreamSynchronize(h->st), "checkpoint");
  });
}

int owt_checkpoint_load(owt_handle *h, const void *host, int64_t bytes) {
  return guard(h, [&] {
    int64_t need = 0;
    owt_checkpoint_bytes(h, &need);
    if (!host || bytes < need) throw OwtError(OWT_ERR_INVALID, "checkpoint image too small");
    CkptHeader hd;
    std::memcpy(&hd, host, sizeof(hd));
    if (std::memcmp(hd.magic, "OWTCKPT1", 8) != 0 || hd.version != 1)
      throw OwtError(OWT_ERR_INVALID, "not a checkpoint image of this library");
    if (hd.NX != h->NX || hd.NY != h->NY || hd.NZ != h->NZ || hd.dt != h->p.dt || hd.dkx != h->p.dkx ||
        hd.dkz != h->p.dkz || hd.alpha_mesh != h->p.alpha_mesh || hd.nu != h->p.nu)
      throw OwtError(OWT_ERR_INVALID, "checkpoint parameters differ from the handle's");
    ck(cudaStreamSynchronize(h->st), "restore");
    ++h->state_version;
    h->drop_graph();
    h->steps = hd.step;
    const long long dstep = (long long)hd.step;
    ck(cudaMemcpyAsync(h->d_step, &dstep, sizeof(dstep), cudaMemcpyHostToDevice, h->st), "H2D");
    const char *o = static_cast<const char *>(host) + sizeof(hd);
    const size_t f = h->fs * sizeof(double2), v = (size_t)h->NY * sizeof(double2);
    for (double2 *ring : {h->v_ring, h->g_ring, h->hv_ring, h->hg_ring, h->q_ring})
      for (int l = 0; l < 3; ++l, o += f)
        ck(cudaMemcpyAsync(h->ring_level(ring, l), o, f, cudaMemcpyHostToDevice, h->st), "H2D");
    for (double2 *fld : {h->u, h->w, h->ox, h->oz, h->lx, h->ly, h->lz}) {
      ck(cudaMemcpyAsync(fld, o, f, cudaMemcpyHostToDevice, h->st), "H2D");
      o += f;
    }
    for (double2 *ring : {h->lxm_ring, h->lzm_ring, h->U_ring, h->W_ring})
      for (int l = 0; l < 3; ++l, o += v)
        ck(cudaMemcpyAsync(ring + (size_t)h->slot(l) * h->NY, o, v, cudaMemcpyHostToDevice, h->st), "H2D");
    for (double *fr : {h->fx_ring, h->fz_ring})
      for (int l = 0; l < 3; ++l, o += sizeof(double))
        ck(cudaMemcpyAsync(fr + h->slot(l), o, sizeof(double), cudaMemcpyHostToDevice, h->st), "H2D");
    h->q_dirty[0] = h->q_dirty[1] = h->q_dirty[2] = false;
    h->initialized = true;
    ck(cudaStreamSynchronize(h->st), "restore");
  });
}

int owt_state_keep(owt_handle *h) {
  return guard(h, [&] {
    if (!h->initialized) throw OwtError(OWT_ERR_STATE, "owt_init_fields (or field uploads) must come first");
    h->recompute_dirty_q();
    if (!h->kept) h->kept = dalloc<double2>(h->image_values(), h->owned);
    h->save_image(h->kept, h->kept_step);
    ck(cudaStreamSynchronize(h->st), "keep state");
  });
}

int owt_state_restore(owt_handle *h) {
  return guard(h, [&] {
    if (!h->kept) throw OwtError(OWT_ERR_STATE, "owt_state_keep must come first");
    ++h->state_version;
    h->load_image(h->kept, h->kept_step);
  });
}

}  // extern "C"

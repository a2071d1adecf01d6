// C ABI of the GPU time step (declared in include/owt_gpu.h): the entry
// points on one handle.  A handle is one channel on one GPU (handle.h); a
// step is the mode kernel with the mean mode beside it, the counter advance,
// the three transform kernels and the nonlinear source, and can be captured
// once as a CUDA graph and replayed.  Batches are in capi_batch.cu,
// checkpoints in capi_checkpoint.cu, the adjoint driver in handle_adjoint.cu.
#include "handle.h"

using namespace owt;

namespace owt {
thread_local std::string g_create_error;
}  // namespace owt

void owt_set_thread_error(const std::string &m) { g_create_error = m; }

extern "C" {

int owt_create(const owt_params *params, owt_handle **out) {
  if (!params || !out) {
    g_create_error = "null argument";
    return OWT_ERR_INVALID;
  }
  *out = nullptr;
  owt_handle *h = new owt_handle();
  try {
    h->setup(*params);
  } catch (const OwtError &e) {
    g_create_error = e.what();
    delete h;
    return e.code;
  } catch (const std::exception &e) {
    g_create_error = e.what();
    delete h;
    return dynamic_cast<const CudaError *>(&e) ? OWT_ERR_CUDA : OWT_ERR_INVALID;
  }
  *out = h;
  return OWT_OK;
}

int owt_destroy(owt_handle *h) {
  delete h;
  return OWT_OK;
}

const char *owt_last_error(const owt_handle *h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int owt_init_fields(owt_handle *h, const double *velx, const double *vely, const double *velz) {
  return guard(h, [&] {
    if (!velx || !vely || !velz) throw OwtError(OWT_ERR_INVALID, "null field");
    ++h->state_version;
    h->init_fields(velx, vely, velz);
    h->sync_and_check();
  });
}

int owt_band_factor_selftest(int kl, int ku, int n, int U, uint64_t seed, int64_t *mismatches, float *ms_thread,
                             float *ms_warp) {
  if (!mismatches || !ms_thread || !ms_warp || n < 1 || U < 1 || !band_supported(kl, ku)) {
    g_create_error = "owt_band_factor_selftest: bad arguments";
    return OWT_ERR_INVALID;
  }
  long long bad = 0;
  if (band_factor_selftest(kl, ku, n, U, seed, &bad, ms_thread, ms_warp) != 0) {
    g_create_error = "owt_band_factor_selftest: CUDA error";
    cudaGetLastError();
    return OWT_ERR_CUDA;
  }
  *mismatches = bad;
  return OWT_OK;
}

int owt_convert_selftest(int64_t n, uint64_t seed, int64_t *counts) {
  if (!counts || n < 0) {
    g_create_error = "owt_convert_selftest: bad arguments";
    return OWT_ERR_INVALID;
  }
  long long c[4] = {};
  if (convert_selftest(n, seed, c) != 0) {
    g_create_error = "owt_convert_selftest: CUDA error";
    cudaGetLastError();
    return OWT_ERR_CUDA;
  }
  for (int k = 0; k < 4; ++k) counts[k] = c[k];
  return OWT_OK;
}

int owt_init_seeded(owt_handle *h, uint64_t seed, double rms) {
  return guard(h, [&] {
    if (!(rms >= 0.0)) throw OwtError(OWT_ERR_INVALID, "rms must be non-negative");
    ++h->state_version;
    h->init_seeded(seed, rms);
    h->sync_and_check();
  });
}

int owt_time_integration(owt_handle *h, int64_t nsteps) {
  return guard(h, [&] {
    if (!h->initialized) throw OwtError(OWT_ERR_STATE, "owt_init_fields (or field uploads) must come first");
    if (nsteps < 0) throw OwtError(OWT_ERR_INVALID, "negative step count");
    ++h->state_version;
    h->run_steps(nsteps);
  });
}

int owt_call(owt_handle *h, int routine) {
  return guard(h, [&] {
    ++h->state_version;
    switch (routine) {
      case OWT_CALL_GET_VOR_FROM_VEL: h->get_vor_from_vel(); break;
      case OWT_CALL_LAMB_VEC: h->lamb_vec(true); break;
      case OWT_CALL_NONLINEAR_SOURCE: h->nonlinear_source(false); break;
      case OWT_CALL_SOLVE_FRICTION_FORCE: h->friction(1); break;
      case OWT_CALL_TIME_INTEGRATION:
        if (!h->initialized) throw OwtError(OWT_ERR_STATE, "owt_init_fields (or field uploads) must come first");
        h->run_steps(1);
        break;
      default: throw OwtError(OWT_ERR_INVALID, "unknown routine id");
    }
    h->check_launch("owt_call");
    h->sync_and_check();
  });
}

int owt_synchronize(owt_handle *h) {
  return guard(h, [&] { h->sync_and_check(); });
}

int owt_get_field(owt_handle *h, int field, double *host) {
  return guard(h, [&] {
    if (!host) throw OwtError(OWT_ERR_INVALID, "null buffer");
    h->to_host(h->field_ptr(field, false), host);
  });
}

int owt_set_field(owt_handle *h, int field, const double *host) {
  return guard(h, [&] {
    if (!host) throw OwtError(OWT_ERR_INVALID, "null buffer");
    ++h->state_version;
    h->to_device(host, h->field_ptr(field, true));
    ck(cudaStreamSynchronize(h->st), "set field");
    h->initialized = true;
  });
}

int owt_get_mean(owt_handle *h, int which, double *host) {
  return guard(h, [&] {
    if (!host) throw OwtError(OWT_ERR_INVALID, "null buffer");
    ck(cudaMemcpyAsync(host, h->mean_ptr(which), h->NY * sizeof(double2), cudaMemcpyDeviceToHost, h->st), "D2H");
    ck(cudaStreamSynchronize(h->st), "D2H");
  });
}

int owt_set_mean(owt_handle *h, int which, const double *host) {
  return guard(h, [&] {
    if (!host) throw OwtError(OWT_ERR_INVALID, "null buffer");
    ++h->state_version;
    ck(cudaMemcpyAsync(h->mean_ptr(which), host, h->NY * sizeof(double2), cudaMemcpyHostToDevice, h->st), "H2D");
    ck(cudaStreamSynchronize(h->st), "H2D");
  });
}

int owt_get_friction(owt_handle *h, double *out6) {
  return guard(h, [&] {
    if (!out6) throw OwtError(OWT_ERR_INVALID, "null buffer");
    double fx[3], fz[3];
    ck(cudaMemcpyAsync(fx, h->fx_ring, sizeof(fx), cudaMemcpyDeviceToHost, h->st), "D2H");
    ck(cudaMemcpyAsync(fz, h->fz_ring, sizeof(fz), cudaMemcpyDeviceToHost, h->st), "D2H");
    h->sync_and_check();
    for (int l = 0; l < 3; ++l) {
      out6[l] = fx[h->slot(l)];
      out6[3 + l] = fz[h->slot(l)];
    }
  });
}

int owt_set_friction(owt_handle *h, const double *in6) {
  return guard(h, [&] {
    if (!in6) throw OwtError(OWT_ERR_INVALID, "null buffer");
    double fx[3], fz[3];
    ++h->state_version;
    for (int l = 0; l < 3; ++l) {
      fx[h->slot(l)] = in6[l];
      fz[h->slot(l)] = in6[3 + l];
    }
    ck(cudaMemcpyAsync(h->fx_ring, fx, sizeof(fx), cudaMemcpyHostToDevice, h->st), "H2D");
    ck(cudaMemcpyAsync(h->fz_ring, fz, sizeof(fz), cudaMemcpyHostToDevice, h->st), "H2D");
    ck(cudaStreamSynchronize(h->st), "H2D");
  });
}

int owt_set_precision(owt_handle *h, int precision) {
  return guard(h, [&] {
    if (precision != OWT_PREC_FP64 && precision != OWT_PREC_MIXED)
      throw OwtError(OWT_ERR_INVALID, "precision must be OWT_PREC_FP64 or OWT_PREC_MIXED");
    if (precision != h->precision) {
      ++h->state_version;
      ck(cudaStreamSynchronize(h->st), "set precision");
      h->drop_graph();
      h->precision = precision;
    }
  });
}

int owt_use_graph(owt_handle *h, int on) {
  return guard(h, [&] {
    ck(cudaStreamSynchronize(h->st), "use graph");
    if (!on) h->drop_graph();
    h->use_graph = on != 0;
  });
}

int owt_get_step(const owt_handle *h, int64_t *step) {
  if (!h || !step) return OWT_ERR_INVALID;
  *step = h->steps;
  return OWT_OK;
}

int owt_get_stream(const owt_handle *h, void **stream) {
  if (!h || !stream) return OWT_ERR_INVALID;
  *stream = (void *)h->st;
  return OWT_OK;
}

int owt_get_launch_count(const owt_handle *h, int64_t *count) {
  if (!h || !count) return OWT_ERR_INVALID;
  *count = h->launches;
  return OWT_OK;
}

int owt_get_grid(const owt_handle *h, double *y) {
  if (!h || !y) return OWT_ERR_INVALID;
  std::memcpy(y, h->grid.y.data(), h->grid.y.size() * sizeof(double));
  return OWT_OK;
}

int owt_statistics(owt_handle *h, double *out7ny) {
  return guard(h, [&] {
    if (!out7ny) throw OwtError(OWT_ERR_INVALID, "null buffer");
    double *d = reinterpret_cast<double *>(h->tmpA);  // 7 NY doubles fit easily
    launch_stats(h->u, h->ring_level(h->v_ring, 0), h->w, h->NY, h->NZ, h->NXH, d, h->st);
    ++h->launches;
    h->check_launch("statistics");
    ck(cudaMemcpyAsync(out7ny, d, 7 * (size_t)h->NY * sizeof(double), cudaMemcpyDeviceToHost, h->st), "D2H");
    h->sync_and_check();
  });
}

int owt_set_option(owt_handle *h, int option, int64_t value) {
  return guard(h, [&] {
    ck(cudaStreamSynchronize(h->st), "set option");
    h->drop_graph();
    if (option == OWT_OPT_FORCE_DENSE_BANDS) {
      h->force_dense = value != 0;
    } else if (option == OWT_OPT_FFT_STOCKHAM) {
      h->fft_stockham = value != 0;
    } else if (option == OWT_OPT_MEAN_SPLIT) {
      h->mean_split = value != 0;
    } else if (option == OWT_OPT_HOST_CHUNKS) {
      if (value < 0 || value > 8) throw OwtError(OWT_ERR_INVALID, "host-step chunks must be within [0, 8]");
      h->host_chunks = (int)value;
    } else if (option == OWT_OPT_MODES_VARIANT) {
      if (value < -1 || value >= modes_variant_count()) throw OwtError(OWT_ERR_INVALID, "no such variant");
      h->forced_variant = (int)value;
    } else {
      throw OwtError(OWT_ERR_INVALID, "unknown option");
    }
  });
}

const char *owt_tuning_report(const owt_handle *h) { return h ? h->tuning.c_str() : ""; }
const char *owt_setup_report(const owt_handle *h) { return h ? h->setup_report.c_str() : ""; }

int owt_get_info(const owt_handle *h, int what, int64_t *value) {
  if (!h || !value) return OWT_ERR_INVALID;
  switch (what) {
    case OWT_INFO_SPARSE_SOLVE: *value = ((h->sparse_v || h->sparse_v6) && !h->force_dense) ? 1 : 0; return OWT_OK;
    case OWT_INFO_PATTERN_VIOLATIONS: *value = h->pattern_violations; return OWT_OK;
    case OWT_INFO_DEVICE_BYTES: *value = (int64_t)h->device_bytes; return OWT_OK;
    case OWT_INFO_MODES_VARIANT: *value = h->forced_variant >= 0 ? h->forced_variant : h->modes_variant; return OWT_OK;
    case OWT_INFO_MODES_VARIANTS: *value = modes_variant_count(); return OWT_OK;
    default: return OWT_ERR_INVALID;
  }
}

int owt_enqueue_stage(owt_handle *h, int stage) {
  return guard(h, [&] {
    if (!h->initialized) throw OwtError(OWT_ERR_STATE, "owt_init_fields must come first");
    switch (stage) {
      case OWT_STAGE_MODES: h->ensure_tuned(); h->stage_modes(); h->launches += 1; break;
      case OWT_STAGE_MEAN: h->stage_mean(); h->launches += 1; break;
      case OWT_STAGE_LAMB: h->launches += launch_lamb(h->xform_args(), h->precision, h->st); break;
      case OWT_STAGE_NONLINEAR: launch_nl(h->nl_args(true), h->st); h->launches += 1; break;
      case OWT_STAGE_ZBACK: case OWT_STAGE_XLAMB: case OWT_STAGE_ZFWD: case OWT_STAGE_MEAN_LAMB:
        launch_lamb_part(h->xform_args(), h->precision, stage - OWT_STAGE_ZBACK, h->st);
        h->launches += 1;
        break;
      default: throw OwtError(OWT_ERR_INVALID, "unknown stage");
    }
    h->check_launch("stage");
  });
}

int owt_set_wall_velocity(owt_handle *h, const double *vw_bottom, const double *vw_top) {
  return guard(h, [&] {
    if (!vw_bottom != !vw_top) throw OwtError(OWT_ERR_INVALID, "give both walls' velocities, or neither");
    ck(cudaStreamSynchronize(h->st), "wall velocity");
    ++h->state_version;
    const bool on = vw_bottom != nullptr;
    if (on) {
      if (!h->vw) h->vw = dalloc<double2>(2 * (size_t)h->M, h->owned);
      const size_t b = (size_t)h->M * sizeof(double2);
      ck(cudaMemcpyAsync(h->vw, vw_bottom, b, cudaMemcpyHostToDevice, h->st), "H2D");
      ck(cudaMemcpyAsync(h->vw + h->M, vw_top, b, cudaMemcpyHostToDevice, h->st), "H2D");
      ck(cudaStreamSynchronize(h->st), "H2D");
    }
    if (on != h->vw_on) h->drop_graph();  // the captured mode kernel holds the pointer
    h->vw_on = on;
  });
}

int owt_get_wall_velocity(owt_handle *h, double *vw_bottom, double *vw_top) {
  return guard(h, [&] {
    if (!vw_bottom || !vw_top) throw OwtError(OWT_ERR_INVALID, "null buffer");
    const size_t b = (size_t)h->M * sizeof(double2);
    if (!h->vw_on) {
      std::memset(vw_bottom, 0, b);
      std::memset(vw_top, 0, b);
      return;
    }
    ck(cudaMemcpyAsync(vw_bottom, h->vw, b, cudaMemcpyDeviceToHost, h->st), "D2H");
    ck(cudaMemcpyAsync(vw_top, h->vw + h->M, b, cudaMemcpyDeviceToHost, h->st), "D2H");
    ck(cudaStreamSynchronize(h->st), "D2H");
  });
}

int owt_dy_apply(owt_handle *h, int order, const double *in, double *out) {
  return guard(h, [&] {
    if (order != 1 && order != 2) throw OwtError(OWT_ERR_INVALID, "order must be 1 or 2");
    if (!in || !out) throw OwtError(OWT_ERR_INVALID, "null buffer");
    h->to_device(in, h->tmpC);
    h->dapply(1, h->tmpC, h->tmpA);
    if (order == 1) {
      launch_combine_y(h->tmpB, h->tmpA, h->c11, nullptr, nullptr, h->NY, h->M, h->st);
    } else {
      h->dapply(2, h->tmpC, h->tmpB);
      launch_combine_y(h->tmpB, h->tmpA, h->c21, h->tmpB, h->c22, h->NY, h->M, h->st);
    }
    ++h->launches;
    h->check_launch("dy apply");
    h->to_host(h->tmpB, out);
  });
}

int owt_time_integration_host(owt_handle *h, const double *const *hist, const double *means, const double *fric,
                              double *vely, double *vory, double *fric_out) {
  return guard(h, [&] {
    if (!hist || !means || !fric || !vely || !vory || !fric_out) throw OwtError(OWT_ERR_INVALID, "null buffer");
    for (int i = 0; i < 12; ++i)
      if (!hist[i]) throw OwtError(OWT_ERR_INVALID, "null history field");
    h->step_host(hist, means, fric, vely, vory, fric_out);
  });
}

int owt_fourier2physical(owt_handle *h, const double *spec, double *phys) {
  return guard(h, [&] {
    if (!spec || !phys) throw OwtError(OWT_ERR_INVALID, "null buffer");
    h->fourier2physical(spec, phys);
  });
}

int owt_physical2fourier(owt_handle *h, const double *phys, double *spec) {
  return guard(h, [&] {
    if (!spec || !phys) throw OwtError(OWT_ERR_INVALID, "null buffer");
    h->physical2fourier(phys, spec);
  });
}

}  // extern "C"

// hmec_graph.cu -- one timestep (sections a1-a19 of cpp/h_mec_rsf_v9.cpp:
// 377-1726) as one CUDA graph launch.
//
// The reference's step is a loop of global (plastic) iterations, each with a
// direct solve; here each solve is an FGMRES whose restart and Arnoldi loops
// end on convergence.  Host-driven, every loop exit is a host look at a
// device flag (a stream drain) and every kernel is a host launch.  In the
// graph the three loops are conditional WHILE nodes: the device kernels that
// end each trip (the global-iteration control of :1310-1457, the FGMRES
// restart decision, the Arnoldi step count) set the loops' conditions, so a
// whole timestep runs from one graph launch with no host round trip, and the
// host reads the device scalars once at the end.
//
// The graph is captured from the same launch code as the host-driven step,
// after one host-driven step has done the lazy set-up (launch shapes, the
// V-cycle pass table).  Every loop is bounded: an Arnoldi trip ends the loop
// or advances the step count (at most krylov_restart per cycle), a restart
// cycle stops or runs an Arnoldi step (at most krylov_maxit per solve), and
// the global loop ends on the reference's exit test, at niterglobal
// iterations (:135), on a non-finite solution, or on its own guard.
#include <cstring>
#include <vector>

#include "hmec_internal.cuh"

namespace {

__global__ void k_graph_begin(GraphCtl* c, int cap, cudaGraphConditionalHandle h) {
    c->gi = 0;
    c->cap = cap;
    cudaGraphSetConditional(h, 1u);
}

// End of a global iteration: the step's Krylov totals, then another
// iteration unless the exit test passed or the solution is not finite.
__global__ void k_gi_cond(DevScalars* ds, GraphCtl* c, cudaGraphConditionalHandle h) {
    ds->krylov_total += ds->krylov_iters;
    ds->krylov_maxrel = fmax(ds->krylov_maxrel, ds->krylov_relres);
    c->gi += 1;
    const int more = !ds->loop_done && !(ds->status & HMEC_DEV_NAN) && c->gi < c->cap;
    cudaGraphSetConditional(h, more ? 1u : 0u);
}

int status_from_device_bits(int bits) {
    if (bits & HMEC_DEV_BOUNDS) return HMEC_ERR_BOUNDS;
    if (bits & HMEC_DEV_NAN) return HMEC_ERR_NAN;
    if (bits & HMEC_DEV_RSF_NOCONV) return HMEC_ERR_RSF_NOCONV;
    if (bits & HMEC_DEV_KRYLOV_NOCONV) return HMEC_ERR_KRYLOV_NOCONV;
    if (bits & HMEC_DEV_TIMEOUT) return HMEC_ERR_TIMEOUT;
    return HMEC_OK;
}

// Ends every capture still open on the context's streams (after a failure
// in the middle of a capture) and clears the sticky capture error.
void abandon_capture(hmec_inst* ctx, cudaStream_t main) {
    cudaStream_t ss[4] = {main, ctx->gr.body[0], ctx->gr.body[1], ctx->gr.body[2]};
    for (cudaStream_t s : ss) {
        if (!s) continue;
        cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(s, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(s, &g);
            if (g && s == main) cudaGraphDestroy(g);
        }
    }
    for (cudaStream_t a : ctx->gs4) {
        if (!a) continue;
        cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(a, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(a, &g);
        }
    }
    if (ctx->up_stream) {
        cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(ctx->up_stream, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(ctx->up_stream, &g);
        }
    }
    for (cudaStream_t a : ctx->sv.aux) {
        cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(a, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(a, &g);
        }
    }
    cudaGetLastError();
}

// Launches one instance's timestep into the capture its stream belongs to,
// ending with the copy of its device scalars to the pinned host mirror;
// records the launch counts of the parts in ctx->gr.
int capture_step(hmec_inst* ctx) {
    GraphState& gs = ctx->gr;
    for (int k = 0; k < 3; k++)
        if (!gs.body[k]) HMEC_CUDA(ctx, cudaStreamCreateWithFlags(&gs.body[k], cudaStreamNonBlocking));
    if (!gs.ctl) HMEC_CUDA(ctx, cudaMalloc(&gs.ctl, sizeof(GraphCtl)));
    const int64_t l_start = ctx->launches;
    cudaStream_t main = ctx->stream;
    int rc = HMEC_OK;
    int64_t n_restart = 0, n_inner = 0, n_global = 0;
    do {
        // a1-a5: the step's status word cleared, markers -> nodes, step begin
        if (cudaMemsetAsync(&ctx->ds->status, 0, sizeof(int), main) != cudaSuccess) {
            rc = HMEC_ERR_CUDA;
            break;
        }
        if ((rc = p2g_run(ctx)) || (rc = markers_stream_issue(ctx)) || (rc = step_begin(ctx))) break;
        cudaGraphConditionalHandle hg = 0;
        if ((rc = graph_handle(ctx, main, &hg))) break;
        HMEC_LAUNCH(ctx, k_graph_begin, 1, 1, 0, gs.ctl, ctx->p.niterglobal + 1, hg);
        if ((rc = graph_while_begin(ctx, main, hg, gs.body[0]))) break;
        const int64_t l0 = ctx->launches;
        {
            // a6-a15: one global iteration
            StreamScope scope(ctx, gs.body[0]);
            if ((rc = iter_prepare(ctx)) || (rc = iter_assemble(ctx)) || (rc = solver_setup(ctx))) break;
            if ((rc = solver_capture_solve(ctx, gs.body[1], gs.body[2], &n_restart, &n_inner))) break;
            if ((rc = iter_finish(ctx))) break;
            HMEC_LAUNCH(ctx, k_gi_cond, 1, 1, 0, ctx->ds, gs.ctl, hg);
        }
        n_global = ctx->launches - l0 - n_restart - n_inner;
        if ((rc = graph_while_end(ctx, gs.body[0]))) break;
        // a16-a19 (and a18/a20 when advection is on)
        if ((rc = step_end(ctx))) break;
        if (ctx->p.advect_markers && (rc = advect_run(ctx))) break;
        if ((rc = markers_stream_join(ctx))) break;
        if (cudaMemcpyAsync(ctx->hs, ctx->ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, main) != cudaSuccess) {
            rc = HMEC_ERR_CUDA;
            break;
        }
    } while (0);
    if (rc == HMEC_OK && cudaGetLastError() != cudaSuccess) rc = HMEC_ERR_CUDA;
    ctx->stream = main;
    gs.n_global = n_global;
    gs.n_restart = n_restart;
    gs.n_inner = n_inner;
    gs.n_top = ctx->launches - l_start - n_global - n_restart - n_inner;
    ctx->launches = l_start;  // the captured launches run when the graph does
    return rc;
}

int build(hmec_inst* ctx) {
    GraphState& gs = ctx->gr;
    cudaStream_t main = ctx->stream;
    HMEC_CUDA(ctx, cudaStreamBeginCapture(main, cudaStreamCaptureModeRelaxed));
    const int rc = capture_step(ctx);
    if (rc != HMEC_OK) {
        abandon_capture(ctx, main);
        return rc;
    }
    cudaGraph_t g = nullptr;
    HMEC_CUDA(ctx, cudaStreamEndCapture(main, &g));
    gs.graph = g;
    HMEC_CUDA(ctx, cudaGraphInstantiate(&gs.exec, g, 0));
    return HMEC_OK;
}

}  // namespace

int graph_handle(hmec_inst* ctx, cudaStream_t s, cudaGraphConditionalHandle* h) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    cudaGraph_t g = nullptr;
    HMEC_CUDA(ctx, cudaStreamGetCaptureInfo(s, &st, nullptr, &g, nullptr, nullptr, nullptr));
    if (st != cudaStreamCaptureStatusActive || !g) {
        ctx->err = "graph_handle: the stream is not capturing";
        return HMEC_ERR_STATE;
    }
    HMEC_CUDA(ctx, cudaGraphConditionalHandleCreate(h, g, 0u, 0u));
    return HMEC_OK;
}

int graph_while_begin(hmec_inst* ctx, cudaStream_t s, cudaGraphConditionalHandle h, cudaStream_t bs) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    HMEC_CUDA(ctx, cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd));
    if (st != cudaStreamCaptureStatusActive || !g) {
        ctx->err = "graph_while_begin: the stream is not capturing";
        return HMEC_ERR_STATE;
    }
    std::vector<cudaGraphNode_t> d(deps, deps + nd);
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    HMEC_CUDA(ctx, cudaGraphAddNode(&node, g, d.empty() ? nullptr : d.data(), nullptr, d.size(), &np));
    cudaGraph_t body = np.conditional.phGraph_out[0];
    HMEC_CUDA(ctx, cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    HMEC_CUDA(ctx, cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    return HMEC_OK;
}

int graph_while_end(hmec_inst* ctx, cudaStream_t bs) {
    cudaGraph_t g = nullptr;
    HMEC_CUDA(ctx, cudaStreamEndCapture(bs, &g));
    return HMEC_OK;
}

int graph_timestep(hmec_inst* ctx, hmec_step_report* rep, bool* used) {
    GraphState& gs = ctx->gr;
    *used = false;
    // host-driven: graphs off, a kernel being timed launch by launch, or the
    // first step (it does the lazy set-up the capture relies on)
    if (!ctx->p.graph || gs.state < 0 || !ctx->prof.name.empty()) return HMEC_OK;
    if (!gs.warm) return HMEC_OK;
    if (gs.state == 0) {
        const int rc = build(ctx);
        if (rc != HMEC_OK) {
            gs.state = -1;
            gs.why = ctx->err;
            ctx->err.clear();
            return HMEC_OK;  // the caller runs the host-driven step
        }
        gs.state = 1;
    }
    HMEC_CUDA(ctx, cudaGraphLaunch(gs.exec, ctx->stream));
    HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *used = true;
    return graph_report(ctx, rep);
}

// The graph copied the device scalars into hs at its end.
int graph_report(hmec_inst* ctx, hmec_step_report* rep) {
    const GraphState& gs = ctx->gr;
    const DevScalars& s = *ctx->hs;
    ctx->launches += gs.n_top + (int64_t)s.iters_in_step * gs.n_global + (int64_t)s.krylov_cycles * gs.n_restart +
                     (int64_t)s.krylov_total * gs.n_inner;
    ctx->in_step = 0;
    const int st = status_from_device_bits(s.status);
    if (rep) {
        rep->timestep = s.timestep - 1;  // the step just completed (the graph advanced the counter)
        rep->global_iters = s.iters_in_step;
        rep->ynlast = s.ynlast + 1;
        rep->krylov_iters = s.krylov_total;
        rep->status = st;
        rep->timesum = s.timesum;
        rep->dt = s.dt;
        rep->Vmax = s.Vmax;
        rep->max_krylov_relres = s.krylov_maxrel;
    }
    if (st != HMEC_OK) {
        ctx->err = "timestep finished with a non-OK status (see report)";
        return st;
    }
    return HMEC_OK;
}

// ------------------------------------------------------------ ensembles
// Every member's step captured side by side: the members' streams fork from
// the context's origin stream and join it again, so the graph holds n
// independent branches, each with its own three conditional loops.
int ensemble_graph_step(hmec_ctx* E, hmec_step_report* reps, bool* used) {
    *used = false;
    const size_t n = E->inst.size();
    if (E->gstate < 0 || n < 2) return HMEC_OK;
    for (hmec_inst* m : E->inst)
        if (!m->p.graph || !m->gr.warm || !m->prof.name.empty() || m->gr.state < 0) return HMEC_OK;
    if (E->gstate == 0) {
        hmec_inst* m0 = E->inst[0];
        auto off = [&](const std::string& why) {
            E->gstate = -1;
            E->why = why;
            return HMEC_OK;
        };
        if (!E->origin && cudaStreamCreateWithFlags(&E->origin, cudaStreamNonBlocking) != cudaSuccess)
            return off("cannot create the ensemble stream");
        if (!E->ev_fork && cudaEventCreateWithFlags(&E->ev_fork, cudaEventDisableTiming) != cudaSuccess)
            return off("cannot create the ensemble events");
        while (E->ev_join.size() < n) {
            cudaEvent_t e = nullptr;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return off("cannot create events");
            E->ev_join.push_back(e);
        }
        if (cudaStreamBeginCapture(E->origin, cudaStreamCaptureModeRelaxed) != cudaSuccess)
            return off("cannot capture the ensemble step");
        int rc = cudaEventRecord(E->ev_fork, E->origin) == cudaSuccess ? HMEC_OK : HMEC_ERR_CUDA;
        for (size_t k = 0; k < n && rc == HMEC_OK; k++) {
            hmec_inst* m = E->inst[k];
            if (cudaStreamWaitEvent(m->stream, E->ev_fork, 0) != cudaSuccess) rc = HMEC_ERR_CUDA;
            if (rc == HMEC_OK) rc = capture_step(m);
            if (rc == HMEC_OK && (cudaEventRecord(E->ev_join[k], m->stream) != cudaSuccess ||
                                  cudaStreamWaitEvent(E->origin, E->ev_join[k], 0) != cudaSuccess))
                rc = HMEC_ERR_CUDA;
            if (rc != HMEC_OK && E->why.empty()) E->why = m->err;
        }
        cudaGraph_t g = nullptr;
        if (rc == HMEC_OK && cudaStreamEndCapture(E->origin, &g) != cudaSuccess) rc = HMEC_ERR_CUDA;
        if (rc == HMEC_OK && cudaGraphInstantiate(&E->exec, g, 0) != cudaSuccess) rc = HMEC_ERR_CUDA;
        if (rc != HMEC_OK) {
            for (hmec_inst* m : E->inst) abandon_capture(m, m->stream);
            cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
            if (cudaStreamIsCapturing(E->origin, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
                cudaGraph_t g2 = nullptr;
                cudaStreamEndCapture(E->origin, &g2);
                if (g2) cudaGraphDestroy(g2);
            }
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            (void)m0;
            return off(E->why.empty() ? "ensemble capture failed" : E->why);
        }
        E->graph = g;
        E->gstate = 1;
    }
    if (cudaGraphLaunch(E->exec, E->origin) != cudaSuccess || cudaStreamSynchronize(E->origin) != cudaSuccess) {
        E->err = "ensemble graph launch failed";
        return HMEC_ERR_CUDA;
    }
    *used = true;
    int first_bad = HMEC_OK;
    for (size_t k = 0; k < n; k++) {
        const int rc = graph_report(E->inst[k], reps ? &reps[k] : nullptr);
        if (rc && !first_bad) first_bad = rc;
    }
    if (first_bad) E->err = "a member's timestep finished with a non-OK status (see its report)";
    return first_bad;
}

void ensemble_graph_free(hmec_ctx* E) {
    if (E->exec) cudaGraphExecDestroy(E->exec);
    if (E->graph) cudaGraphDestroy(E->graph);
    if (E->ev_fork) cudaEventDestroy(E->ev_fork);
    for (cudaEvent_t e : E->ev_join) cudaEventDestroy(e);
    if (E->origin) cudaStreamDestroy(E->origin);
    E->exec = nullptr;
    E->graph = nullptr;
    E->ev_fork = nullptr;
    E->ev_join.clear();
    E->origin = nullptr;
}

void graph_free(hmec_inst* ctx) {
    GraphState& gs = ctx->gr;
    if (gs.exec) cudaGraphExecDestroy(gs.exec);
    if (gs.graph) cudaGraphDestroy(gs.graph);
    for (int k = 0; k < 3; k++)
        if (gs.body[k]) cudaStreamDestroy(gs.body[k]);
    cudaFree(gs.ctl);
    gs = GraphState();
}

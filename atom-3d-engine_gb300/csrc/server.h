// server.h — the served form: a request loop with continuous batching on one GPU.
//
// Client threads submit render requests; one worker thread owns all device work. Scene tapes
// (and their payloads: SDF volumes, GI probes) stay resident across requests; a request either
// names a resident scene (a camera update) or brings a new scene, optionally with a mesh to
// bake into one of its volumes first (bakes are cached by mesh content). Requests are admitted
// against an HBM budget (resident scenes + the pass-sequence slots + every admitted frame's
// device and pinned staging); a request that does not fit waits until completed frames free
// memory, least-recently-used idle scenes are dropped from the device (their host copy stays
// and is recompiled on demand). Admitted requests are coalesced in arrival order into pass
// sequences (BatchEngine waves) on `max_inflight` slots, each with its own stream and
// buffers, so requests arriving while others are on the GPU start as soon as a slot frees
// and their work overlaps on the device. In plain mode the worker instead renders one
// request at a time through the per-frame launch sequence (the baseline the batched form is
// measured against).
#pragma once
#include <condition_variable>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch.h"
#include "capi_internal.h"

namespace mm3e {

class Server;

}  // namespace mm3e

struct mm3e_server {
    std::unique_ptr<mm3e::Server> impl;
};

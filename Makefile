# Harness targets and knobs of the reference Makefile, building the harness mains
# in gcq_gb300/harness/ against libgcq.so (sm_103a) instead of compiling each
# harness with hipcc.  Same variable names and defaults; QUEUE selects the queue at
# compile time (-DUSE_GWFQ ...), as the reference does.
#
#   make tb QUEUE=gwfq TB_RUN_MS=1000 TB_WARMUP_MS=200 TB_CHUNK_OPS=128
#   make hist QUEUE=sfq HIST_THREADS=64 HIST_OPS=16
#   make bfs QUEUE=gwfq BFS_GEN="--grid 4096 4096 --keep 0.6 --diag 0.01 --seed 2"
#   make bfs QUEUE=glfq BFS_GRAPH=graphs/road_usa.mtx
#   make rt QUEUE=gwfq SCENE=1 THREADS=1024 BOUNCES=4
#   make rt-compact SCENE=2 BOUNCES=12      (the stream-compaction baseline)
#   make rt-bench QUEUE=gwfq SCENE=0 THREADS=1024 BOUNCES=4   (benchmark scenes, 1024x1024)
#
# The linearizability checker is test infrastructure here (oracle/), run by the
# test suite rather than by a make target.

CXX ?= g++
PYTHON ?= python3
LIB_DIR := gcq_gb300/_build
HARNESS := gcq_gb300/harness

RT_BUILD_DIR ?= out
TB_BUILD_DIR ?= out
HIST_BUILD_DIR ?= out
BFS_BUILD_DIR ?= out

# Raytracing (RT) args
QUEUE ?= gwfq
SCENE ?= 0
THREADS ?= 1024
BOUNCES ?= 4
GPU_NAME ?=

# Throughput-benchmark args
TB_FIFO_MODE ?= 0
TB_RUN_MS ?= 500
TB_WARMUP_MS ?= 100
TB_CHUNK_OPS ?= 64
TB_BLOCK_SIZE ?= 256
TB_FIFO_OPS_PER_THREAD ?= 64
TB_ONLY_BALANCED ?= 0
TB_ONLY_SPLIT ?= 0
TB_CSV_FILE ?= benchmark_results.csv
TB_EXTRA_FLAGS ?=

# History generator args
HIST_THREADS ?= 64
HIST_OPS ?= 16
HIST_MODE ?= 0
HIST_PRODUCER_PERCENT ?= 50
HIST_BLOCK_SIZE ?= 256
HIST_OUT_DIR ?= out/histories
HIST_EXTRA_FLAGS ?=

# BFS args (BFS_GEN, when set, generates the graph instead of reading BFS_GRAPH)
BFS_GRAPH_DIR ?= graphs
BFS_GRAPH ?= $(BFS_GRAPH_DIR)/delaunay_n21.mtx
BFS_GEN ?=
BFS_THREADS ?= 8192
BFS_BLOCK ?= 256
BFS_SRC_VERTEX ?= 0
BFS_ITERS ?= 10
BFS_WARMUP ?= 3
BFS_PERSISTENT ?= 0
BFS_EXTRA_FLAGS ?=
BFS_CSV_NAME ?= bfs_bench_final.csv

# Compile-time args
QUEUE_N ?= 32768
EXTRA_FLAGS ?=

ifeq ($(QUEUE),gwfq)
QUEUE_DEF := -DUSE_GWFQ
else ifeq ($(QUEUE),glfq)
QUEUE_DEF := -DUSE_GLFQ
else ifeq ($(QUEUE),wfq)
QUEUE_DEF := -DUSE_WFQ
else ifeq ($(QUEUE),sfq)
QUEUE_DEF := -DUSE_SFQ
else
$(error Unsupported QUEUE='$(QUEUE)'. Use one of: gwfq glfq wfq sfq)
endif

RT_BIN := $(RT_BUILD_DIR)/rt_$(QUEUE)
TB_BIN := $(TB_BUILD_DIR)/tb_$(QUEUE)_fifo$(TB_FIFO_MODE)
HIST_BIN := $(HIST_BUILD_DIR)/history_$(QUEUE)
HIST_JSONL := $(HIST_OUT_DIR)/history_$(QUEUE)_m$(HIST_MODE)_t$(HIST_THREADS)_o$(HIST_OPS).jsonl
BFS_BIN := $(BFS_BUILD_DIR)/bfs_$(QUEUE)

HXX = $(CXX) -O2 -std=c++17 -Iinclude -I$(HARNESS) $(QUEUE_DEF)
HLINK = -L$(LIB_DIR) -lgcq -Wl,-rpath,$(abspath $(LIB_DIR)) -pthread

.PHONY: all lib rt rt-build rt-run rt-bench rt-bench-build rt-bench-run rt-compact rt-compact-build rt-compact-run tb tb-build tb-run tb-build-fifo tb-run-fifo hist hist-build hist-run \
        hist-run-all bfs bfs-build bfs-build-all bfs-run bfs-sweep clean

all: rt

# libgcq.so: every CUDA translation unit for sm_103a (incremental)
lib:
	$(PYTHON) -c "import sys; sys.path.insert(0, '.'); from gcq_gb300 import build; build.build()"

rt: rt-run

rt-build: lib
	@mkdir -p $(RT_BUILD_DIR)
	@echo "[RT] Building $(RT_BIN) (queue=$(QUEUE), qN=$(QUEUE_N))"
	$(HXX) -DRT_QUEUE_N=$(QUEUE_N) $(EXTRA_FLAGS) $(HARNESS)/rt.cpp -o $(RT_BIN) $(HLINK)

rt-run: rt-build
	@echo "[RT] Running $(RT_BIN) scene=$(SCENE) bounces=$(BOUNCES) threads=$(THREADS)"
	GPU_NAME="$(GPU_NAME)" $(RT_BIN) $(SCENE) $(BOUNCES) $(THREADS)

rt-bench: rt-bench-run

rt-bench-build: lib
	@mkdir -p $(RT_BUILD_DIR)
	@echo "[RT] Building $(RT_BUILD_DIR)/rt_bench_$(QUEUE) (benchmark scenes, qN=$(QUEUE_N))"
	$(HXX) -DRT_QUEUE_N=$(QUEUE_N) $(EXTRA_FLAGS) $(HARNESS)/rt_bench.cpp -o $(RT_BUILD_DIR)/rt_bench_$(QUEUE) $(HLINK)

rt-bench-run: rt-bench-build
	GPU_NAME="$(GPU_NAME)" $(RT_BUILD_DIR)/rt_bench_$(QUEUE) $(SCENE) $(BOUNCES) $(THREADS)

rt-compact: rt-compact-run

rt-compact-build: lib
	@mkdir -p $(RT_BUILD_DIR)
	@echo "[RT] Building $(RT_BUILD_DIR)/rt_compact (stream-compaction baseline)"
	$(HXX) $(EXTRA_FLAGS) $(HARNESS)/rt_compact.cpp -o $(RT_BUILD_DIR)/rt_compact $(HLINK)

rt-compact-run: rt-compact-build
	GPU_NAME="$(GPU_NAME)" $(RT_BUILD_DIR)/rt_compact $(SCENE) $(BOUNCES)

tb: tb-run

tb-build: lib
	@mkdir -p $(TB_BUILD_DIR)
	@echo "[TB] Building $(TB_BIN) (queue=$(QUEUE), fifo_mode=$(TB_FIFO_MODE))"
	$(HXX) -DRUN_MS=$(TB_RUN_MS) -DWARMUP_MS=$(TB_WARMUP_MS) -DCHUNK_OPS=$(TB_CHUNK_OPS) \
		-DBLOCK_SIZE=$(TB_BLOCK_SIZE) -DONLY_BALANCED=$(TB_ONLY_BALANCED) -DONLY_SPLIT=$(TB_ONLY_SPLIT) \
		-DMODE_FIFO=$(TB_FIFO_MODE) -DFIFO_OPS_PER_THREAD=$(TB_FIFO_OPS_PER_THREAD) \
		-DCSV_FILE=\"$(TB_CSV_FILE)\" $(TB_EXTRA_FLAGS) $(HARNESS)/tb.cpp -o $(TB_BIN) $(HLINK)

tb-run: tb-build
	@echo "[TB] Running $(TB_BIN)"
	GPU_NAME="$(GPU_NAME)" $(TB_BIN)

tb-build-fifo: TB_FIFO_MODE=1
tb-build-fifo: tb-build

tb-run-fifo: TB_FIFO_MODE=1
tb-run-fifo: tb-run

hist: hist-run

hist-build: lib
	@mkdir -p $(HIST_BUILD_DIR)
	@echo "[HIST] Building $(HIST_BIN) (queue=$(QUEUE))"
	$(HXX) -DHIST_THREADS=$(HIST_THREADS) -DHIST_OPS=$(HIST_OPS) -DHIST_MODE=$(HIST_MODE) \
		-DHIST_PRODUCER_PERCENT=$(HIST_PRODUCER_PERCENT) -DHIST_BLOCK_SIZE=$(HIST_BLOCK_SIZE) \
		$(HIST_EXTRA_FLAGS) $(HARNESS)/history.cpp -o $(HIST_BIN) $(HLINK)

hist-run: hist-build
	@mkdir -p $(HIST_OUT_DIR)
	@echo "[HIST] Writing $(HIST_JSONL)"
	$(HIST_BIN) $(HIST_JSONL) $(HIST_THREADS) $(HIST_OPS) $(HIST_MODE) $(HIST_PRODUCER_PERCENT)

hist-run-all:
	@for q in gwfq glfq wfq sfq; do \
		echo "[HIST] queue=$$q"; \
		$(MAKE) --no-print-directory hist-run QUEUE=$$q HIST_THREADS=$(HIST_THREADS) HIST_OPS=$(HIST_OPS) \
			HIST_MODE=$(HIST_MODE) HIST_PRODUCER_PERCENT=$(HIST_PRODUCER_PERCENT) \
			HIST_BLOCK_SIZE=$(HIST_BLOCK_SIZE) HIST_OUT_DIR=$(HIST_OUT_DIR) \
			HIST_EXTRA_FLAGS='$(HIST_EXTRA_FLAGS)' || exit 1; \
	done

bfs: bfs-run

bfs-build: lib
	@mkdir -p $(BFS_BUILD_DIR)
	@echo "[BFS] Building $(BFS_BIN) (queue=$(QUEUE))"
	$(HXX) $(BFS_EXTRA_FLAGS) $(HARNESS)/bfs.cpp -o $(BFS_BIN) $(HLINK)

bfs-build-all:
	@for q in gwfq glfq wfq sfq; do \
		$(MAKE) --no-print-directory bfs-build QUEUE=$$q BFS_BUILD_DIR='$(BFS_BUILD_DIR)' \
			BFS_EXTRA_FLAGS='$(BFS_EXTRA_FLAGS)' || exit 1; \
	done

bfs-run: bfs-build
	@if [ -z "$(BFS_GEN)" ] && [ ! -f "$(BFS_GRAPH)" ]; then \
		echo "[BFS] graph not found: $(BFS_GRAPH) (set BFS_GEN to generate one)"; \
		exit 2; \
	fi
	@echo "[BFS] Running $(BFS_BIN) threads=$(BFS_THREADS) block=$(BFS_BLOCK)"
	CSV_NAME=$(BFS_CSV_NAME) GPU_NAME="$(GPU_NAME)" $(BFS_BIN) \
		$(if $(BFS_GEN),$(BFS_GEN),--graph "$(BFS_GRAPH)") \
		--threads "$(BFS_THREADS)" --block "$(BFS_BLOCK)" --src "$(BFS_SRC_VERTEX)" \
		--iters "$(BFS_ITERS)" --warmup "$(BFS_WARMUP)" --persistent "$(BFS_PERSISTENT)"

# The sweep of concurrent_bfs/run_bfs_sweep.sh: every queue x thread count x graph,
# one log per point, rows appended to BFS_CSV_NAME.  BFS_GRAPHS lists .mtx/SNAP files
# (relative to BFS_GRAPH_DIR); left empty it sweeps the two generated grids.
BFS_QUEUES ?= gwfq glfq wfq sfq
BFS_CHUNKS ?= 512 1024 2048 4096 8192
BFS_GRAPHS ?=
BFS_LOG_DIR ?= out/bfs_logs
BFS_GPU_FAMILY ?= gb300
BFS_GEN_GRAPHS := gridA:--grid 4096 4096 --keep 0.6 --diag 0.01 --seed 2|gridB:--grid 212 212 --keep 0.6 --diag 0.01 --seed 2

bfs-sweep: bfs-build-all
	@mkdir -p $(BFS_LOG_DIR)
	@set -e; \
	if [ -n "$(BFS_GRAPHS)" ]; then \
		specs=""; for g in $(BFS_GRAPHS); do \
			case "$$g" in /*) p="$$g" ;; *) p="$(BFS_GRAPH_DIR)/$$g" ;; esac; \
			specs="$$specs|$$(basename $$g):--graph $$p"; done; specs="$${specs#|}"; \
	else specs="$(BFS_GEN_GRAPHS)"; fi; \
	IFS='|'; for spec in $$specs; do \
		name="$${spec%%:*}"; args="$${spec#*:}"; \
		for q in $(BFS_QUEUES); do for t in $(BFS_CHUNKS); do \
			log="$(BFS_LOG_DIR)/bfs_$${q}_$(BFS_GPU_FAMILY)_$${name}_$${t}.log"; \
			echo "[BFS] $$q $$name threads=$$t -> $$log"; \
			IFS=' '; CSV_NAME=$(BFS_CSV_NAME) GPU_NAME="$(GPU_NAME)" $(BFS_BUILD_DIR)/bfs_$$q $$args \
				--threads $$t --block $(BFS_BLOCK) --src $(BFS_SRC_VERTEX) --iters $(BFS_ITERS) \
				--warmup $(BFS_WARMUP) --persistent $(BFS_PERSISTENT) > "$$log" 2>&1 || echo "[BFS] failed, see $$log"; \
			IFS='|'; \
		done; done; \
	done

clean:
	rm -rf out

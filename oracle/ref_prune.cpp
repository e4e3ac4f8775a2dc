// ref_prune — TEST INFRASTRUCTURE ONLY.
//
// Runs two of the reference's rank-0 graph passes on a merged graph given as
// a -d file (contigGraph.txt): recvBufDistNodeGraph (graph.cpp:845-896), then
// masterTipsRemoval (graph.cpp:2194-2265) and masterLowCoverageEdgeRemoval
// (graph.cpp:2267-2300), writing the graph with the reference's own
// gatherDistNodeGraph (graph.cpp:576-696, nodes in the node map's iteration
// order — the order both passes visit them in) before, after the tips pass and
// after the low-coverage pass. graph.cpp is compiled in through the include
// below (its main() renamed); nothing of it is copied here.
// Usage: ref_prune -k K -c C -i contigGraph.txt -o <new dir>
// (writes <dir>/before.txt, <dir>/tips.txt, <dir>/lowcov.txt).
#define main swap_reference_main
#include "graph.cpp"
#undef main

static void dump(distNodeGraph *g, parameter *p, MPIEnviroment *mpi, const char *name) {
    char *buf = g->gatherDistNodeGraph(p, mpi);
    std::string path = std::string(p->outputPath) + "/" + name;
    FILE *fp = fopen(path.c_str(), "w");
    fprintf(fp, "%s\n", buf);
    fclose(fp);
    delete[] buf;
}

int main(int argc, char *argv[]) {
    MPIEnviroment MPIcontrol;
    MPIcontrol.init(argc, argv);
    parameter parameters;
    parameters.getParameters(argc, argv, &MPIcontrol);

    FILE *in = fopen(parameters.fastaPath, "rb");
    if (!in) {
        printf("cannot open %s\n", parameters.fastaPath);
        return 1;
    }
    fseek(in, 0, SEEK_END);
    long n = ftell(in);
    fseek(in, 0, SEEK_SET);
    char *rBuf = new char[n + 1];  // released by recvBufDistNodeGraph
    if (fread(rBuf, 1, n, in) != (size_t)n) {
        printf("short read\n");
        return 1;
    }
    fclose(in);
    rBuf[n] = 0;

    distNodeGraph *nodeGraph = new distNodeGraph(&parameters, &MPIcontrol);
    nodeGraph->recvBufDistNodeGraph(rBuf, &parameters, &MPIcontrol);
    dump(nodeGraph, &parameters, &MPIcontrol, "before.txt");
    nodeGraph->masterTipsRemoval(&parameters, &MPIcontrol);
    dump(nodeGraph, &parameters, &MPIcontrol, "tips.txt");
    nodeGraph->masterLowCoverageEdgeRemoval(&parameters, &MPIcontrol);
    dump(nodeGraph, &parameters, &MPIcontrol, "lowcov.txt");
    MPIcontrol.finalize();
    return 0;
}

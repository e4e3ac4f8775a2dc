// ref_simplify — TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's masterSimplifyNodeGraph (graph.cpp:2089-2192) once on
// a merged graph given as gathered node lines (a -d file, or the output of a
// tip / low-coverage pass): recvBufDistNodeGraph (graph.cpp:845-896), the
// graph written with the reference's own gatherDistNodeGraph (graph.cpp:
// 576-696: node map order, the order the pass visits), the pass, the graph
// written again. graph.cpp is compiled in through the include below (its
// main() renamed); nothing of it is copied here.
// Usage: ref_simplify -k K -c C -i lines.txt -o <new dir>
// (writes <dir>/before.txt, <dir>/after.txt).
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
    nodeGraph->masterSimplifyNodeGraph(&parameters, &MPIcontrol);
    dump(nodeGraph, &parameters, &MPIcontrol, "after.txt");
    MPIcontrol.finalize();
    return 0;
}

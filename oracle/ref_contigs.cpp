// ref_contigs — TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own rank-0 contig stage on a merged graph given as a
// -d file (contigGraph.txt, the gatherDistNodeGraph layout): the call
// sequence of the reference main() after the gather (graph.cpp:3629-3683):
// recvBufDistNodeGraph, masterSimplifyNodeGraph, printContigs, four rounds of
// tip / low-coverage / bubble removal with simplification, cross-edge
// removal, masterPrintContigs. Lets the tests feed the GPU merge's output to
// the reference's downstream stages. graph.cpp is compiled in through the
// include below (its main() renamed); nothing of it is copied here.
// Usage: ref_contigs -k K -c C -i contigGraph.txt -o <new dir>
// (writes <dir>/noCEcontigs.fasta and <dir>/CEContig.fasta).
#define main swap_reference_main
#include "graph.cpp"
#undef main

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
    nodeGraph->masterSimplifyNodeGraph(&parameters, &MPIcontrol);
    nodeGraph->printContigs(&parameters, &MPIcontrol);
    for (int i = 0; i < 4; i++) {
        nodeGraph->masterTipsRemoval(&parameters, &MPIcontrol);
        nodeGraph->masterSimplifyNodeGraph(&parameters, &MPIcontrol);
        nodeGraph->masterLowCoverageEdgeRemoval(&parameters, &MPIcontrol);
        nodeGraph->masterSimplifyNodeGraph(&parameters, &MPIcontrol);
        nodeGraph->masterLoopBubbleRemoval(&parameters, &MPIcontrol);
        nodeGraph->masterMultipleEdgeBubbleRemoval(&parameters, &MPIcontrol);
        nodeGraph->masterSimplifyNodeGraph(&parameters, &MPIcontrol);
        nodeGraph->masterGraphStatistic(&parameters, &MPIcontrol);
    }
    nodeGraph->masterRemoveCrossEdge(&parameters, &MPIcontrol);
    nodeGraph->masterPrintContigs(&parameters, &MPIcontrol);
    MPIcontrol.finalize();
    return 0;
}
